"""Block timeline of one time step (diagnostics build).

    python fwi2dacoustic-mpi-lbfgs_gb300/timeline.py [--workload c2] [--nshots 64] [--nt 201] [--step 100]

Builds the engine with FWI_TIMELINE into libfwigpu_timeline.so next to the
product library (which stays untouched), runs one gradient of the workload in
a child process with the timeline armed at --step, and prints, for the
backward and the forward step of that index and per kernel class: the items
(blocks, or general tiles x shots), the first start, last start and last end
(microseconds from the step's first block) and the median item duration; then
the number of items of each class active in every 20 microsecond bin.  It
shows how the general-tile classes and the interior tiles of a step share the
GPU over time.  Needs a GPU.
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys
import tempfile

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
TL_ITEMS = 1 << 16          # TL_ITEMS of csrc/fwi_kernels.cuh
NAMES = ["interior", "z-general", "x-general", "corners"]


def child(args):
    sys.path.insert(0, PKG)
    import fwigpu
    import workloads
    cfgkw, vtrue, vstart, shots = workloads.build(args.workload, nshots=args.nshots, nt=args.nt)
    e = fwigpu.Engine(fwigpu.make_config(**cfgkw, use_graph=1))
    e.set_shots(shots)
    e.set_model(vtrue)
    obs = e.forward()
    e.set_observed(obs)
    e.set_model(vstart)
    e.gradient()
    e.close()                                   # writes the timeline


def report(path):
    a = np.fromfile(path, dtype=np.uint64).reshape(8, TL_ITEMS, 2).astype(np.int64)
    for direction, base in (("backward", 0), ("forward", 4)):
        live = [np.where((a[base + c, :, 0] != 0) & (a[base + c, :, 1] != 0))[0] for c in range(4)]
        if not any(len(v) for v in live):
            continue
        t0 = min(a[base + c, v, 0].min() for c, v in enumerate(live) if len(v))
        print(f"{direction} step:")
        end = 0
        for c, v in enumerate(live):
            if not len(v):
                continue
            st, en = a[base + c, v, 0] - t0, a[base + c, v, 1] - t0
            end = max(end, en.max())
            print(f"  {NAMES[c]:10s} items {len(v):6d}  first start {st.min() / 1e3:7.1f} us  last start "
                  f"{st.max() / 1e3:7.1f}  last end {en.max() / 1e3:7.1f}  "
                  f"median item {np.median(en - st) / 1e3:6.2f} us")
        bins = np.arange(0, end + 20000, 20000)
        print("  items active per 20 us bin (" + " / ".join(NAMES) + "):")
        for b0, b1 in zip(bins[:-1], bins[1:]):
            row = []
            for c, v in enumerate(live):
                st, en = a[base + c, v, 0] - t0, a[base + c, v, 1] - t0
                row.append(int(np.sum((st < b1) & (en > b0))) if len(v) else 0)
            print(f"   {b0 / 1e3:6.0f} us: " + " ".join(f"{n:6d}" for n in row))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="c2")
    ap.add_argument("--nshots", type=int, default=64)
    ap.add_argument("--nt", type=int, default=201)
    ap.add_argument("--step", type=int, default=100)
    ap.add_argument("--child", action="store_true", help=argparse.SUPPRESS)
    args = ap.parse_args()
    if args.child:
        child(args)
        return
    sys.path.insert(0, PKG)
    import build
    lib = build.build(defines=("FWI_TIMELINE",), out=os.path.join(PKG, "libfwigpu_timeline.so"))
    with tempfile.TemporaryDirectory() as d:
        out = os.path.join(d, "timeline.bin")
        env = dict(os.environ, FWI_LIB=lib, FWI_TIMELINE_STEP=str(args.step), FWI_TIMELINE_OUT=out)
        subprocess.run([sys.executable, os.path.abspath(__file__), "--child", "--workload", args.workload,
                        "--nshots", str(args.nshots), "--nt", str(args.nt), "--step", str(args.step)],
                       env=env, check=True)
        report(out)


if __name__ == "__main__":
    main()
