"""The quality-study arithmetic (host only): relMSE with the reference's own
variance removed is unbiased, and the summary renders."""
import numpy as np

from lisa_gb300 import study


def test_reference_variance_correction_is_unbiased():
    rng = np.random.default_rng(0)
    truth = rng.uniform(0.1, 2.0, (64, 64, 3))
    sd = 0.5 * truth
    n_x, n_ref = 16, 64
    x = truth + rng.normal(size=truth.shape) * sd / np.sqrt(n_x)
    ref = truth + rng.normal(size=truth.shape) * sd / np.sqrt(n_ref)
    exact = study.relmse(x, truth)
    raw = study.relmse(x, ref)
    corrected = study.relmse(x, ref, (sd ** 2) / n_ref)
    # the raw figure is inflated by about n_x / n_ref; the corrected one is not
    assert raw > exact * 1.1
    assert abs(corrected - exact) < 0.1 * exact


def test_summary_renders():
    row = {"study": "hard_indirect", "estimator": "compat", "scene": "s", "triangles": 10, "res": 8, "spp": 4,
           "reference": {"spp": 64, "seconds": 1.0},
           "plain": {"ms": 1.0, "rays": 1e6, "relmse": 0.2, "relmse_corrected": 0.1},
           "guided": {"ms": 1.1, "rays": 1e6, "relmse": 0.1, "relmse_corrected": 0.05},
           "equal_time_relmse": {"plain": 0.1, "guided": 0.055}, "time_to_plain_error": 0.55}
    md = study.summary_md([row], "cmd")
    assert "| guided | 1.1 |" in md and "0.550" in md
