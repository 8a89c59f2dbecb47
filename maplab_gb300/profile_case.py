"""Runs one configuration of the bundle adjuster for profiling (ncu, or the
CUDA-event times it prints).

    # the evaluation kernel alone, L2 flushed before each launch
    python -m maplab_gb300.profile_case visual --config c2 --block 64 --min-blocks 3 --launches 3
    # one solve
    python -m maplab_gb300.profile_case solve --config c4 --precision mixed --precond learned --iters 6
    # the same after autotuning, with only the solve inside the profiler range
    # (ncu --profile-from-start off)
    python -m maplab_gb300.profile_case solve --config c4 --autotune --profile-range
"""
import argparse
import ctypes
import json

from . import _native as N
from . import ba, synth


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("what", choices=["visual", "solve"])
    ap.add_argument("--config", default="c2")
    ap.add_argument("--block", type=int, default=0)
    ap.add_argument("--min-blocks", type=int, default=0)
    ap.add_argument("--launches", type=int, default=3)
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="mixed")
    ap.add_argument("--precond", choices=["jacobi", "chain", "learned"], default="learned")
    ap.add_argument("--iters", type=int, default=6)
    ap.add_argument("--pcg", type=int, default=25)
    ap.add_argument("--autotune", action="store_true")
    ap.add_argument("--device-loop", type=int, default=1)
    ap.add_argument("--reject-every", type=int, default=0)
    ap.add_argument("--reproj", type=int, default=0)
    ap.add_argument("--schur-split", type=int, default=0, help="1: two threads per Schur chunk, 2: one")
    ap.add_argument("--pcg-product", type=int, default=0, help="1: read-once product, 2: both rows")
    ap.add_argument("--chain-segment", type=int, default=0, help="segmented sweeps (positions per block) or 1")
    ap.add_argument("--profile-range", action="store_true",
                    help="cuProfilerStart / cuProfilerStop around the solve only")
    a = ap.parse_args()
    m = synth.generate(a.config)
    with ba.BundleAdjuster(m.desc) as g:
        if a.block or a.min_blocks:
            g.set_tuning(visual_block=a.block, visual_min_blocks=a.min_blocks)
        prec = N.MBA_PRECISION_MIXED if a.precision == "mixed" else N.MBA_PRECISION_FP64
        if a.autotune:
            print(json.dumps({"tuning": g.autotune(prec)}))
        # explicit settings override the autotuner's choice
        if a.schur_split or a.pcg_product or a.chain_segment:
            g.set_tuning(schur_split=a.schur_split, pcg_product=a.pcg_product, chain_segment=a.chain_segment)
        if a.what == "visual":
            ms = g.time_visual_kernel(mode=1 if prec == N.MBA_PRECISION_MIXED else 0, iters=a.launches)
            print(json.dumps({"visual_ms_per_launch": ms, "observations": m.desc.num_observations}))
            return
        pre = {"jacobi": N.MBA_PRECOND_BLOCK_JACOBI, "chain": N.MBA_PRECOND_CHAIN,
               "learned": N.MBA_PRECOND_LEARNED}[a.precond]
        model = None
        if pre == N.MBA_PRECOND_LEARNED:
            from . import train_preconditioner as TP
            model = TP.load_default_model()
            g.set_preconditioner_model(model)
        opts = ba.default_options(max_num_iterations=a.iters, max_linear_iterations=a.pcg, precision=prec,
                                  preconditioner=pre, check_tolerances=0, use_cuda_graph=2 if a.device_loop else 1,
                                  reject_outliers_every_n_iters=a.reject_every,
                                  outlier_use_reprojection_error=a.reproj)
        cuda = ctypes.CDLL("libcuda.so.1") if a.profile_range else None
        if cuda is not None:
            cuda.cuProfilerStart()
        s = g.solve(opts)
        if cuda is not None:
            cuda.cuProfilerStop()
        st = g.stats()
        print(json.dumps({"iterations": s["num_iterations"] - 1, "final_cost": s["final_cost"],
                          "time_ms": s["iterations"][-1]["time_ms"], "pcg": s["linear_iterations"],
                          "keyframes": st["num_keyframes"], "observations": st["num_observations"],
                          "device_bytes": st["device_bytes"], "schur_pose_blocks": st["num_schur_pose_blocks"]}))
        if model is not None:
            model.close()


if __name__ == "__main__":
    main()
