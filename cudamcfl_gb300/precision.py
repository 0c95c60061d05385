"""Single- vs double-precision error of the transport kernel.

The engine transports photons in FP32 (exact-IEEE or fast-math builds) and
tallies in 64-bit integers.  The FP64 build of the same kernel
(MATH_F64) runs every position, direction, step and probability in double
on the same photon streams, so a run of each on identical seeds isolates the
error that single precision adds.  Photon k of a run draws the same random
numbers in every build; the paths agree until a rounding difference flips a
discrete decision (a Fresnel or roulette draw, a voxel boundary) and then
decorrelate, so the comparison is statistical: B batches with different
seeds, every batch run in every build, and the per-batch differences
(paired) give the mean error and its standard error.

Reported per build against FP64: integrated R, T and absorbed fractions
(relative difference and paired z), and for the R/T images and the
photon-hitting density the relative RMS difference over the pixels/voxels
with signal and the share of them beyond 3 paired standard errors.

    python -m cudamcfl_gb300.precision --photons 1e9 --batches 10

runs the large precision-study medium (media.config5: 512 x 512 x 256
voxels, mu_s' = 20/cm, wide-field source); --small uses its quarter
resolution variant, --exact-stepping runs every build with voxel-boundary
stepping.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np
from scipy.stats import t as _t

from . import MATH_EXACT, MATH_F64, MATH_FAST, SOURCE_WIDEFIELD, Context, run_desc
from . import media as media_mod

ONE = float(2**32 - 1)  # the tally unit: weight of one launched photon
MODES = {"fast": MATH_FAST, "exact": MATH_EXACT, "f64": MATH_F64}


def _paired(a: np.ndarray, b: np.ndarray):
    """Mean and standard error over batches (axis 0) of a - b."""
    d = a - b
    n = d.shape[0]
    return d.mean(axis=0), d.std(axis=0, ddof=1) / np.sqrt(n)


def _block_sum(fhd: np.ndarray, shape, block: int) -> np.ndarray:
    """Photon hitting density summed over block^3 voxel cubes (the grid's
    extents must be multiples of block)."""
    nz, ny, nx = shape
    if block <= 1:
        return fhd.astype(np.float64)
    v = fhd.reshape(nz // block, block, ny // block, block, nx // block, block)
    return v.sum(axis=(1, 3, 5), dtype=np.float64).ravel()


def study(ctx: Context, med, rd_for_seed, batches: int, modes=("fast", "exact", "f64"), fluence: bool = True,
          fluence_block: int = 1):
    """Runs every build on the same B seeds; returns the per-build batch
    arrays {mode: {"R": (B, pix), "T": ..., "phd": (B, cells), "A": (B,),
    "Rall": (B,), "Tall": (B,), "seconds": float, "steps": int}}; the photon
    hitting density is kept summed over fluence_block^3 voxel cells."""
    out = {m: {"R": [], "T": [], "phd": [], "A": [], "Rall": [], "Tall": [], "seconds": 0.0, "steps": 0,
               "photons": 0} for m in modes}
    old = ctx.get_option("math")
    try:
        for b in range(batches):
            rd = rd_for_seed(1000 + 7 * b)
            for mode in modes:
                ctx.set_option("math", MODES[mode])
                t0 = time.perf_counter()
                r = ctx.run(med, rd, images=False, raw=True, fluence=fluence, emission128=False)
                out[mode]["seconds"] += time.perf_counter() - t0
                n = float(rd.photons)
                se = r.stats_exc
                out[mode]["R"].append(r.Rd.astype(np.float64) / (ONE * n))
                out[mode]["T"].append(r.Tt.astype(np.float64) / (ONE * n))
                if fluence and r.fhd is not None:
                    out[mode]["phd"].append(_block_sum(r.fhd, med.shape, fluence_block) / (ONE * n))
                out[mode]["A"].append(se["absorbed"] / (ONE * n))
                out[mode]["Rall"].append(se["exit_top"] / (ONE * n))
                out[mode]["Tall"].append(se["exit_bottom"] / (ONE * n))
                out[mode]["steps"] += int(se["steps"])
                out[mode]["photons"] += int(rd.photons)
    finally:
        ctx.set_option("math", old)
    for mode in modes:
        for k in ("R", "T", "phd", "A", "Rall", "Tall"):
            out[mode][k] = np.asarray(out[mode][k])
    return out


def _field(a: np.ndarray, b: np.ndarray, floor: float = 0.0):
    """Relative RMS difference and paired z statistics of two (B, n) tallies
    over the entries whose mean exceeds floor."""
    mean_b = b.mean(axis=0)
    keep = mean_b > floor
    if not keep.any():
        return {"entries": 0}
    d, se = _paired(a[:, keep], b[:, keep])
    ok = se > 0
    z = np.zeros_like(d)
    z[ok] = d[ok] / se[ok]
    rel = d / mean_b[keep]
    # with B batches the paired z follows Student's t with B-1 degrees of
    # freedom: the 3-sigma gate at its 0.27 % two-sided tail
    thr = float(_t.isf(0.0027 / 2, max(1, a.shape[0] - 1)))
    return {"entries": int(keep.sum()), "rel_rms": float(np.sqrt(np.mean(rel * rel))),
            "rel_mean": float(np.mean(rel)), "beyond_3se": float(np.mean(np.abs(z[ok]) > 3.0)) if ok.any() else 0.0,
            "t_threshold": thr, "beyond_t": float(np.mean(np.abs(z[ok]) > thr)) if ok.any() else 0.0,
            "max_abs_z": float(np.max(np.abs(z[ok]))) if ok.any() else 0.0,
            "mean_z": float(np.mean(z[ok])) if ok.any() else 0.0}


def _scalar(a: np.ndarray, b: np.ndarray):
    d, se = _paired(a, b)
    m = float(b.mean())
    return {"value": float(a.mean()), "f64": m, "rel_diff": float(d / m) if m else 0.0,
            "paired_se_rel": float(se / m) if m else 0.0, "z": float(d / se) if se > 0 else 0.0}


def summarize(res: dict, ref: str = "f64", min_photons: float = 20.0) -> dict:
    """Per build against `ref`: integrated fractions, and the R/T images and
    fluence over the entries holding at least min_photons photons' weight
    per batch."""
    out = {}
    for mode, r in res.items():
        if mode == ref:
            continue
        b = res[ref]
        pix_floor = min_photons / max(1, r["photons"] // len(r["A"]))
        out[mode] = {
            "R_total": _scalar(r["Rall"], b["Rall"]), "T_total": _scalar(r["Tall"], b["Tall"]),
            "absorbed": _scalar(r["A"], b["A"]),
            "R_image": _field(r["R"], b["R"], pix_floor), "T_image": _field(r["T"], b["T"], pix_floor),
        }
        if r["phd"].size and b["phd"].size:
            out[mode]["fluence"] = _field(r["phd"], b["phd"], pix_floor)
        out[mode]["steps_ratio"] = r["steps"] / max(1, b["steps"])
    out["timing"] = {m: {"seconds": r["seconds"], "photons": r["photons"],
                         "photons_per_s": r["photons"] / r["seconds"] if r["seconds"] else None,
                         "steps_per_photon": r["steps"] / max(1, r["photons"])} for m, r in res.items()}
    return out


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--photons", type=float, default=1e8, help="photons per build in total (split over batches)")
    ap.add_argument("--batches", type=int, default=10)
    ap.add_argument("--small", action="store_true", help="the 128 x 128 x 64 variant at 0.04 cm")
    ap.add_argument("--modes", default="fast,exact,f64")
    ap.add_argument("--no-fluence", action="store_true")
    ap.add_argument("--exact-stepping", action="store_true", help="voxel-boundary stepping in every build")
    args = ap.parse_args(argv)
    m = media_mod.config5(shape=(64, 128, 128), voxel=0.04) if args.small else media_mod.config5()
    ctx = Context(device=0)
    med = ctx.medium(m.labels, m.bulks, voxel_cm=m.voxel_cm, fluor_map=m.fluor_map)
    per_batch = int(args.photons) // args.batches
    w, h = m.info["widefield"]

    def rd_for_seed(seed):
        return run_desc(per_batch, det=m.det, fluence=0 if args.no_fluence else 1, seed_exc=seed, seed_fl=seed + 1,
                        kind=SOURCE_WIDEFIELD, width=w, height=h, exact_stepping=1 if args.exact_stepping else 0)

    # full size: the fluence compared on 4^3-voxel cells (128 x 128 x 64)
    res = study(ctx, med, rd_for_seed, args.batches, tuple(args.modes.split(",")), fluence=not args.no_fluence,
                fluence_block=1 if args.small else 4)
    s = summarize(res)
    s["workload"] = {"medium": "config5" + (" quarter resolution" if args.small else ""),
                     "shape_zyx": list(m.labels.shape), "voxel_cm": m.voxel_cm[0], "photons_per_build": per_batch *
                     args.batches, "batches": args.batches, "source": f"wide-field {w:.2f} x {h:.2f} cm",
                     "fluence_cells": "voxels" if args.small else "4x4x4-voxel cells",
                     "stepping": "voxel boundary" if args.exact_stepping else "the reference's"}
    print(json.dumps(s), flush=True)
    med.free()
    ctx.close()
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
