"""Image-quality studies: guided vs plain sampling at equal time, against a
high-spp reference accumulated in FP64 on the GPU.

  python -m lisa_gb300.study hard_indirect [--res 1024] [--spp 256] [--ref-spp 16384] [--estimator physical]
  python -m lisa_gb300.study batch [--n 64] [--spp-scale 1] [--ref-mult 16] [--estimator physical]

relMSE = mean over pixels and channels of (x - ref)^2 / (ref^2 + 1e-2).
Because the reference has finite spp, E[(x - ref)^2] = MSE(x) + Var(ref);
the "corrected" figure subtracts the reference's own per-pixel variance of
the mean (its FP64 sample variance / its spp), which leaves an unbiased
estimate of the render's relMSE.  Equal time: Monte Carlo error falls as
1/spp, so a render that took t_g for relMSE e_g reaches e_g * t_g / t_p in the
plain render's time t_p; "time to plain's error" is (t_g / t_p) * (e_g / e_p).

Each run prints one JSON line per measurement and, with --summary, writes a
short markdown table.
"""
from __future__ import annotations

import argparse
import json
import sys
import time
from typing import List

import numpy as np

from . import scenes as S


def relmse(x: np.ndarray, ref: np.ndarray, ref_var_of_mean: np.ndarray = None) -> float:
    d2 = (np.asarray(x, np.float64) - ref) ** 2
    if ref_var_of_mean is not None:
        d2 = d2 - ref_var_of_mean
    return float(np.mean(d2 / (ref * ref + 1e-2)))


def _render(L, params, **opt):
    r = L.Renderer(params, L.default_options(stage_timing=1, **opt))
    t0 = time.perf_counter()
    st = r.render()
    wall = time.perf_counter() - t0
    return r, st, wall


def _estimator(L, args) -> int:
    return L._native.LISA_ESTIMATOR_PHYSICAL if args.estimator == "physical" else L._native.LISA_ESTIMATOR_COMPAT


def hard_indirect(args) -> List[dict]:
    import lisa_gb300 as L

    sc = S.hard_indirect(level=args.level, width=args.res, height=args.res, num_samples=args.spp,
                         num_bounces=8)
    out = []
    # reference: plain sampling, FP64 accumulation, progressive launches
    p_ref = L.params_from_scene(sc, num_samples=args.ref_spp)
    est = _estimator(L, args)
    ref = L.Renderer(p_ref, L.default_options(accum_fp64=1, seed=1000003, estimator=est))
    t0 = time.perf_counter()
    done = 0
    while done < args.ref_spp:
        k = min(args.ref_chunk, args.ref_spp - done)
        ref.render_progressive(k)
        done += k
    ref_s = time.perf_counter() - t0
    _, var, R = ref.image(variance=True, fp64=True)
    vom = var / args.ref_spp
    ref.close()
    p = L.params_from_scene(sc)
    rows = {}
    for name, opt in (("plain", dict(seed=12)), ("guided", dict(seed=13, mode=L._native.LISA_MODE_GUIDED))):
        r, st, wall = _render(L, p, estimator=est, **opt)
        img = r.image()
        rows[name] = dict(ms=st.ms_device, wall_s=wall, rays=st.rays, relmse=relmse(img, R),
                          relmse_corrected=relmse(img, R, vom), guide_loss=st.guide_loss,
                          stages_ms={"trace": st.ms_trace, "shade": st.ms_shade, "nee": st.ms_nee,
                                     "guide": st.ms_guide, "other": st.ms_other},
                          guide_infer={"ms": st.ms_guide_infer, "rows": st.guide_infer_rows},
                          guide_train={"ms": st.ms_guide_train, "samples": st.guide_train_samples},
                          launches=st.launches_total)
        r.close()
    tp, tg = rows["plain"]["ms"], rows["guided"]["ms"]
    ep, eg = rows["plain"]["relmse_corrected"], rows["guided"]["relmse_corrected"]
    out.append({
        "study": "hard_indirect", "estimator": args.estimator, "scene": sc.name, "triangles": sc.num_triangles,
        "res": args.res,
        "spp": args.spp, "bounces": 8, "reference": {"spp": args.ref_spp, "accum": "fp64", "seconds": ref_s},
        "plain": rows["plain"], "guided": rows["guided"],
        "equal_time_relmse": {"plain": ep, "guided": eg * tg / tp},
        "time_to_plain_error": (tg / tp) * (eg / ep) if ep > 0 else None,
    })
    return out


def batch(args) -> List[dict]:
    import lisa_gb300 as L

    G = L._native.LISA_MODE_GUIDED
    scs = S.batch_scenes(n=args.n, seed=5, max_res=args.max_res)
    spp = [max(4, int(round(s.num_samples * args.spp_scale))) for s in scs]
    params = [L.params_from_scene(s, num_samples=k) for s, k in zip(scs, spp)]
    est = _estimator(L, args)
    tune_p = L.autotune(params, cache=args.cache, estimator=est)
    tune_g = L.autotune(params, cache=args.cache, mode=G, estimator=est)
    res = {}
    imgs = {}
    for name, tune, opt in (("plain", tune_p, dict(seed=12, estimator=est)),
                            ("guided", tune_g, dict(seed=13, mode=G, estimator=est))):
        o = L.apply_tuning(tune, L.default_options(stage_timing=1, **opt))
        r = L.Renderer(params, o)
        r.render()  # warm-up: graph capture, guide training from scratch below
        r.close()
        r = L.Renderer(params, o)
        t0 = time.perf_counter()
        st = r.render()
        wall = time.perf_counter() - t0
        res[name] = dict(ms=st.ms_device, wall_s=wall, rays=st.rays, mrays_per_s=st.rays / st.ms_device / 1e3,
                         launches=st.launches_total, tuning=tune.as_dict(),
                         stages_ms={"trace": st.ms_trace, "shade": st.ms_shade, "nee": st.ms_nee,
                                    "guide": st.ms_guide, "other": st.ms_other},
                         guide_infer={"ms": st.ms_guide_infer, "rows": st.guide_infer_rows},
                         guide_train={"ms": st.ms_guide_train, "samples": st.guide_train_samples})
        imgs[name] = [r.image(k) for k in range(len(params))]
        r.close()
    # per-scene reference: ref_mult x the spp, plain, FP64
    p_ref = [L.params_from_scene(s, num_samples=k * args.ref_mult) for s, k in zip(scs, spp)]
    t0 = time.perf_counter()
    ref = L.Renderer(p_ref, L.apply_tuning(tune_p, L.default_options(accum_fp64=1, seed=1000003, estimator=est)))
    ref.render()
    ref_s = time.perf_counter() - t0
    scenes_out = []
    tp, tg = res["plain"]["ms"], res["guided"]["ms"]
    # Scenes under guide_min_spp render on the plain path in the guided batch
    # too, at the plain batch's cost; the guided batch's extra time belongs
    # to the guided scenes.  Attributing it to them in proportion to their
    # paths (and their plain time to their share of all paths) gives each
    # guided scene the time ratio 1 + (tg/tp - 1) * paths / guided paths.
    min_spp = L.default_options().guide_min_spp
    paths = [s.width * s.height * k for s, k in zip(scs, spp)]
    guided_paths = sum(pp for pp, k in zip(paths, spp) if k >= min_spp)
    r_guided = 1.0 + (tg / tp - 1.0) * sum(paths) / max(guided_paths, 1)
    for k, s in enumerate(scs):
        _, var, R = ref.image(k, variance=True, fp64=True)
        vom = var / (spp[k] * args.ref_mult)
        ep = relmse(imgs["plain"][k], R, vom)
        eg = relmse(imgs["guided"][k], R, vom)
        guided = spp[k] >= min_spp
        ratio = r_guided if guided else 1.0
        scenes_out.append({"scene": s.name, "triangles": s.num_triangles, "res": [s.width, s.height],
                           "spp": spp[k], "bounces": s.num_bounces, "relmse_plain": ep, "relmse_guided": eg,
                           "equal_time_guided": eg * tg / tp, "guided": guided, "time_ratio_attributed": ratio,
                           "equal_time_guided_attributed": eg * ratio})
    ref.close()
    g_rows = [x for x in scenes_out if x["guided"] and x["relmse_plain"] > 0]
    return [{
        "study": "batch", "estimator": args.estimator, "scenes": len(scs), "spp_scale": args.spp_scale,
        "total_paths": int(sum(s.width * s.height * k for s, k in zip(scs, spp))),
        "reference": {"spp_mult": args.ref_mult, "accum": "fp64", "seconds": ref_s},
        "plain": res["plain"], "guided": res["guided"], "per_scene": scenes_out,
        "median_equal_time_ratio": float(np.median([x["equal_time_guided"] / max(x["relmse_plain"], 1e-30)
                                                    for x in scenes_out])),
        "guide_min_spp": int(min_spp), "guided_scenes": len(g_rows), "time_ratio_guided_scenes": r_guided,
        "median_equal_time_ratio_guided_scenes": float(np.median(
            [x["equal_time_guided_attributed"] / x["relmse_plain"] for x in g_rows])) if g_rows else None,
        "median_equal_spp_ratio_guided_scenes": float(np.median(
            [x["relmse_guided"] / x["relmse_plain"] for x in g_rows])) if g_rows else None,
    }]


def summary_md(rows: List[dict], cmd: str) -> str:
    lines = [f"Command: `{cmd}`", ""]
    for r in rows:
        if r["study"] == "hard_indirect":
            lines += [f"## hard indirect, {r['estimator']} estimator ({r['scene']}, {r['triangles']:,} tris, "
                      f"{r['res']}^2, {r['spp']} spp)", "",
                      f"Reference: {r['reference']['spp']} spp plain, FP64 accumulation "
                      f"({r['reference']['seconds']:.0f} s).", "",
                      "| method | device ms | Mrays | relMSE | relMSE (ref. variance removed) |",
                      "|---|---|---|---|---|"]
            for m in ("plain", "guided"):
                x = r[m]
                lines.append(f"| {m} | {x['ms']:.1f} | {x['rays'] / 1e6:.0f} | {x['relmse']:.6g} | "
                             f"{x['relmse_corrected']:.6g} |")
            lines += ["", f"Equal-time relMSE: plain {r['equal_time_relmse']['plain']:.6g}, guided "
                          f"{r['equal_time_relmse']['guided']:.6g}; guided time to plain's error = "
                          f"{r['time_to_plain_error']:.3f} x plain's time.", ""]
        else:
            lines += [f"## batch of {r['scenes']} scenes, {r['estimator']} estimator (spp x {r['spp_scale']}, "
                      f"{r['total_paths']:,} paths)", "",
                      "| method | device ms | Mrays/s | launches | tuning | stage ms |", "|---|---|---|---|---|---|"]
            for m in ("plain", "guided"):
                x = r[m]
                t = x["tuning"]
                sm = x.get("stages_ms", {})
                lines.append(f"| {m} | {x['ms']:.1f} | {x['mrays_per_s']:.0f} | {x['launches']} | "
                             f"W={t['paths_in_flight']}, {t['threads_per_block']} thr, refill {t['refill_idle']} | "
                             + ", ".join(f"{k} {v:.0f}" for k, v in sm.items()) + " |")
            gi, gt = r["guided"].get("guide_infer"), r["guided"].get("guide_train")
            if gi and gt:
                lines += ["", f"Guide in the guided batch: inference {gi['ms']:.0f} ms over {gi['rows']:,} vertices, "
                              f"training {gt['ms']:.0f} ms over {gt['samples']:,} samples."]
            lines += ["", f"Median over scenes of guided equal-time relMSE / plain relMSE, every scene "
                          f"charged the batch-wide time ratio {r['guided']['ms'] / r['plain']['ms']:.3f}: "
                          f"{r['median_equal_time_ratio']:.3f}", ""]
            if r.get("median_equal_time_ratio_guided_scenes") is not None:
                lines += [f"The {r['guided_scenes']} guided scenes (spp >= {r['guide_min_spp']}; the others render "
                          f"plain in both batches), the guided batch's extra time attributed to them by their "
                          f"paths (time ratio {r['time_ratio_guided_scenes']:.3f}): median equal-time relMSE "
                          f"ratio {r['median_equal_time_ratio_guided_scenes']:.3f}; at equal spp "
                          f"{r['median_equal_spp_ratio_guided_scenes']:.3f}.", ""]
            lines += ["| scene | tris | res | spp | bounces | guided | relMSE plain | relMSE guided | "
                      "guided at equal time (batch ratio) | (attributed) |",
                      "|---|---|---|---|---|---|---|---|---|---|"]
            for s in r["per_scene"]:
                lines.append(f"| {s['scene']} | {s['triangles']:,} | {s['res'][0]}x{s['res'][1]} | {s['spp']} | "
                             f"{s['bounces']} | {'yes' if s.get('guided') else 'no'} | {s['relmse_plain']:.4g} | "
                             f"{s['relmse_guided']:.4g} | {s['equal_time_guided']:.4g} | "
                             f"{s.get('equal_time_guided_attributed', float('nan')):.4g} |")
            lines.append("")
    return "\n".join(lines) + "\n"


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m lisa_gb300.study")
    sub = ap.add_subparsers(dest="which", required=True)
    h = sub.add_parser("hard_indirect")
    h.add_argument("--res", type=int, default=1024)
    h.add_argument("--level", type=int, default=8)
    h.add_argument("--spp", type=int, default=256)
    h.add_argument("--ref-spp", type=int, default=16384)
    h.add_argument("--ref-chunk", type=int, default=256)
    b = sub.add_parser("batch")
    b.add_argument("--n", type=int, default=64)
    b.add_argument("--max-res", type=int, default=1024)
    # at a fraction of the scenes' spp fewer of them reach guide_min_spp
    b.add_argument("--spp-scale", type=float, default=1.0)
    b.add_argument("--ref-mult", type=int, default=16)
    b.add_argument("--cache", default=None, help="autotuner cache (JSON)")
    for p in (h, b):
        p.add_argument("--summary", default=None, help="write a markdown summary here")
        p.add_argument("--estimator", default="compat", choices=["compat", "physical"])
    args = ap.parse_args(argv)
    rows = hard_indirect(args) if args.which == "hard_indirect" else batch(args)
    for r in rows:
        print(json.dumps(r), flush=True)
    if args.summary:
        with open(args.summary, "w") as f:
            f.write(summary_md(rows, "python -m lisa_gb300.study " + " ".join(argv or sys.argv[1:])))


if __name__ == "__main__":
    main()
