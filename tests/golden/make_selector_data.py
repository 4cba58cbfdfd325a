"""Measures the plan-selector dataset ``selector_timings.npz`` on a GPU.

    python tests/golden/make_selector_data.py [--n 2000] [--out tests/golden/selector_timings.npz]

For each of ``n`` seeded shapes from ``heffte_gb300.selector.sample_shapes``
(sides 32..768, 80% with factors 2, 3, 5 only and 20% with a factor 7 or 11;
c2c / r2c / DCT-II; float / double; at most 2^26 elements) it times the
forward transform of all 16 candidate plans (use_reorder x kernel family x
tile size x radix order) with CUDA events, median of 5 runs after one warm-up,
and stores the features, the times and the shapes.  Progress is kept in
``<out>.partial.npz`` so an interrupted run resumes.
"""
from __future__ import annotations

import argparse
import os
import sys
import time

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", ".."))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=2000)
    ap.add_argument("--seed", type=int, default=2000)
    ap.add_argument("--out", default=os.path.join(os.path.dirname(os.path.abspath(__file__)), "selector_timings.npz"))
    args = ap.parse_args()
    import torch
    from heffte_gb300 import selector
    shapes = selector.sample_shapes(args.n, seed=args.seed)
    t0 = time.time()
    X, T = selector.measure(shapes, path=args.out + ".partial.npz", reps=5,
                            log=lambda m: print(f"{m}  ({time.time() - t0:.0f} s)", flush=True))
    np.savez_compressed(args.out, X=X.astype(np.float32), T=T,
                        sizes=np.array([s for s, _, _ in shapes], dtype=np.int32),
                        kinds=np.array([k for _, k, _ in shapes], dtype=np.int32),
                        precs=np.array([p for _, _, p in shapes], dtype=np.int32),
                        seed=args.seed, device=torch.cuda.get_device_name(0))
    os.remove(args.out + ".partial.npz")
    print(f"wrote {args.out}: {len(X)} shapes in {time.time() - t0:.0f} s")


if __name__ == "__main__":
    main()
