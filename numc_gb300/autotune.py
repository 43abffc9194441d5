"""Autotuner for grouped float32 GEMM plans (run on a GB300).

For every size class of (M, N, K) — classes <=32, <=64, ..., <=1024 — time
one plan of identical problems on each kernel variant (the split GEMM from
scaled float16 planes with 128-column tiles or with 64-column tiles, each
with K cut into 1, 2 or 4 slices whose partial sums a reduction pass adds
in K order; CUDA-core FMA) and record the fastest variant and its slice
count in numc_gb300/autotune_table.txt, which plans read at creation (for
both split plane formats).

    python -m numc_gb300.autotune [--out PATH]

With --clusters it measures the other axis instead: the split GEMM kernel
(scaled float16 planes) as clusters of two CTAs sharing 256 x 256 tiles
(cta_group::2) against single CTAs on 256-column tiles, on square and
long-K problems of the grouped plans' sizes, GEMM kernel time only (CUDA
events around the kernel), and writes numc_gb300/cluster_table.txt.
"""
import argparse
import os
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPRESENTATIVE = [24, 48, 96, 192, 384, 768]        # one size per class 0..5
# (table variant, K slices, name, algo, plan param); 7 = SPLIT_FP16, 1 = SIMT
VARIANTS = [(0, 1, "split128", 7, 128), (0, 2, "split128k2", 7, 2128),
            (0, 4, "split128k4", 7, 4128), (1, 1, "split64", 7, 64),
            (1, 2, "split64k2", 7, 2064), (1, 4, "split64k4", 7, 4064), (2, 1, "simt", 1, 0)]


def time_plan(nc, torch, problems, algo, param, reps=5):
    plan = nc.GemmPlan(problems, algo, param)
    plan.run(graph=True)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        plan.run(graph=True)
    e1.record()
    torch.cuda.synchronize()
    plan.free()
    return e0.elapsed_time(e1) / reps


CLUSTER_SHAPES = [(256, 256, 256), (256, 256, 1024), (512, 512, 512), (512, 512, 1024),
                  (768, 768, 768), (1024, 1024, 1024), (1024, 256, 1024), (256, 1024, 1024),
                  (2048, 2048, 2048)]


def _time_gemm_kernels():
    """Child process: GEMM-kernel milliseconds per shape (phase timing)."""
    import torch
    import numc_gb300 as nc
    out = {}
    for M, N, K in CLUSTER_SHAPES:
        a = torch.randn(M, K, device="cuda")
        b = torch.randn(K, N, device="cuda")
        c = torch.empty(M, N, device="cuda")
        ws = torch.empty(nc.workspace_size("float32", 7, 0, M, K, N), dtype=torch.uint8,
                         device="cuda")
        for _ in range(3):
            nc.gemm(a, b, c, algo=7, workspace=ws)
        torch.cuda.synchronize()
        nc.phase_timing(True)
        for _ in range(20):
            nc.gemm(a, b, c, algo=7, workspace=ws)
        _, gemm_ms, calls = nc.phase_times()
        nc.phase_timing(False)
        out[f"{M}x{N}x{K}"] = gemm_ms / calls
    nc.check_status()
    print(repr(out))


def clusters(path):
    import ast
    import subprocess
    import sys
    res = {}
    for ctas in (2, 1):
        env = dict(os.environ, NUMC_CUDA_SPLIT_CTAS=str(ctas))
        r = subprocess.run([sys.executable, "-m", "numc_gb300.autotune", "--child"], env=env,
                           capture_output=True, text=True, check=True)
        res[ctas] = ast.literal_eval(r.stdout.strip().splitlines()[-1])
    import torch
    lines = ["# split GEMM kernel (scaled float16 planes), GEMM kernel time in ms:",
             "# ctas=2: clusters of two CTAs on 256 x 256 tiles (cta_group::2);",
             "# ctas=1: single CTAs on 128 x 256 tiles.  MxNxK  ctas=2  ctas=1  faster",
             f"# device: {torch.cuda.get_device_name()}, {time.strftime('%Y-%m-%d')}"]
    for key in res[2]:
        t2, t1 = res[2][key], res[1][key]
        lines.append(f"{key} {t2:.4f} {t1:.4f} {2 if t2 < t1 else 1}")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
    print("\n".join(lines))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=None)
    ap.add_argument("--clusters", action="store_true")
    ap.add_argument("--child", action="store_true", help=argparse.SUPPRESS)
    args = ap.parse_args()
    if args.child:
        return _time_gemm_kernels()
    if args.clusters:
        return clusters(args.out or os.path.join(HERE, "cluster_table.txt"))
    args.out = args.out or os.path.join(HERE, "autotune_table.txt")
    import torch
    import numc_gb300 as nc
    lines = ["# grouped float32 GEMM autotune table: mclass nclass kclass variant splits",
             "# classes: 0 <=32, 1 <=64, 2 <=128, 3 <=256, 4 <=512, 5 <=1024",
             "# variants: 0 split GEMM (scaled float16 planes) 128-column tiles,",
             "#           1 the same with 64-column tiles, 2 CUDA-core FMA;",
             "# splits: K slices of the tensor-core variants (k2, k4 below: 2, 4 slices);",
             "# times are ms per plan run (graph replay)",
             f"# device: {torch.cuda.get_device_name()}, {time.strftime('%Y-%m-%d')}"]
    t0 = time.time()
    for cm, M in enumerate(REPRESENTATIVE):
        for cn, N in enumerate(REPRESENTATIVE):
            for ck, K in enumerate(REPRESENTATIVE):
                count = int(np.clip(2.0 ** 32 / (2.0 * M * N * K), 8, 1024))
                a = torch.randn(count, M, K, device="cuda")
                b = torch.randn(count, K, N, device="cuda")
                c = torch.empty(count, M, N, device="cuda")
                problems = [(a[i], b[i], c[i]) for i in range(count)]
                times = {name: time_plan(nc, torch, problems, algo, param)
                         for _, _, name, algo, param in VARIANTS}
                best = min(VARIANTS, key=lambda v: times[v[2]])
                lines.append(f"{cm} {cn} {ck} {best[0]} {best[1]}   # {M}x{N}x{K} x{count}: " +
                             " ".join(f"{k}={v:.3f}" for k, v in times.items()))
                del a, b, c
    with open(args.out, "w") as f:
        f.write("\n".join(lines) + "\n")
    print(f"wrote {args.out} in {time.time() - t0:.0f} s")


if __name__ == "__main__":
    main()
