"""Complex128 receivers of the 96-system bench workload: the accuracy fixture of the
batched mixed-precision path.

The plain complex128 solver (csem_solve_batch_host with precision 64: the reference's
BiCGStab + LU-SGS recurrences, solver.c:93-178 and fdfd.c:287-510, with the reference's
point arithmetic; it matches the reference's own receivers to 1.5e-11 at 1.25 Hz on this
model) solves a subset of the Marlim-shaped batch (synthetic.marlim_like(seed=0)) to
tol = 1e-8/f with the iteration limit raised to `--niter` (the reference's 1000 stops
short of convergence at 0.125 and 0.25 Hz). The subset covers all six frequencies and
the sources `--sources` (default 0, 7 and 15: both ends and the middle of the line).

Runs on a GPU. Writes an npz with
  freqs [nsys], isrc [nsys], rec [nsys][3][nrec] (complex128 Ex, Ey, Ez),
  iters [nsys], status [nsys] (strings), relres [nsys], niter, tol.
The committed copy lives at tests/golden/marlim_like_96/fp64_receivers.npz.

  python tests/golden/make_fp64_receivers.py --out gpurun_out/fp64_receivers.npz
"""
from __future__ import annotations

import argparse
import os
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    ap.add_argument("--niter", type=int, default=4000)
    ap.add_argument("--sources", default="0,7,15")
    ap.add_argument("--freqs", default="", help="comma list (default: the workload's six)")
    args = ap.parse_args()
    import demo_matrixfree_csem_gb300 as cs
    from demo_matrixfree_csem_gb300 import synthetic
    cfg = synthetic.workload("marlim_like_96")
    freqs = [float(f) for f in (args.freqs or cfg.params["freqs"]).split(",")]
    isrc = [int(s) for s in args.sources.split(",")]
    with tempfile.TemporaryDirectory() as d:
        jobs, keep = [], []
        for s in isrc:
            G = synthetic.build_grid(cfg, d)
            ctx = cs.Ctx(G, int(cfg.params["airbc"]), 0)
            keep.append((G, ctx))
            jobs.append(dict(ctx=ctx, freqs=np.asarray(freqs, np.float32),
                             srcs=np.repeat(cfg.acq.src[s:s + 1, :3], len(freqs), axis=0), rec=cfg.acq.rec,
                             precision=64, algopt=1, preco=1, niter=args.niter, tol=1e-8))
    t0 = time.time()
    # one context per source, solved concurrently (one host thread and stream each)
    res = cs.solve_batches(jobs)
    wall = time.time() - t0
    F, S, R, IT, ST, RR = [], [], [], [], [], []
    for s, r in zip(isrc, res):
        for q, f in enumerate(freqs):
            F.append(f)
            S.append(s)
            R.append(r["dcal"][q])
            IT.append(int(r["iters"][q]))
            ST.append(r["status"][q])
            RR.append(float(r["relres"][q]))
            print(f"source {s} {f} Hz: {r['status'][q]} after {int(r['iters'][q])} iterations "
                  f"(relres {r['relres'][q]:.3e})", flush=True)
    os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
    np.savez_compressed(args.out, freqs=np.asarray(F, np.float32), isrc=np.asarray(S, np.int32),
                        rec=np.asarray(R, np.complex128), iters=np.asarray(IT, np.int32), status=np.asarray(ST),
                        relres=np.asarray(RR), niter=args.niter, tol=1e-8, wall_s=wall)
    print(f"wrote {args.out}: {len(F)} systems in {wall:.0f} s")


if __name__ == "__main__":
    main()
