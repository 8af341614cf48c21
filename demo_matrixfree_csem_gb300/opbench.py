"""Operator micro-benchmark: time A, LU-SGS or A-phi applications on a batch of systems.

    python -m demo_matrixfree_csem_gb300.opbench --workload marlim_like_96 --op lusgs \
        --prec 32 --nsys 16 --reps 5 [--schedule pipelined|diagonal] [--vw 0|1|2|4] \
        [--split 1|0] [--overlap 1|0] [--cap N] [--systems 1|2|4] [--lines N] [--tiled 0|1] \
        [--by 4|8|16] [--ctas N]

The schedule flags set the context options of the same names (lusgs_split, lusgs_overlap,
lusgs_cap, lusgs_systems, lusgs_lines, lusgs_tiled, stencil_by, stencil_ctas); the
defaults are the library's. All systems of one call share one frequency (--freq), so the
grouped schedules see full groups.

--op csr compares the matrix-free operator with the same operator assembled in CSR and
applied by cuSPARSE (csem_csr_compare), on the workload's grid without the airwave (the
assembled operator has no airwave coupling), one system.

Vectors are random and stay on the device; each repetition applies the operator to all
systems once through the device-pointer C ABI (csem_*_apply_dev) on the context's
stream, timed with CUDA events on that stream. Prints one JSON line: milliseconds per
application and per system, and the algorithmic HBM rate (bytes per system per
application: A 40/20 B per unknown, LU-SGS 96/48 B per unknown of the LU-SGS grid, in
complex128/complex64). With --reps 1 --warmup 0 it is a small, fixed launch sequence for
profilers.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import tempfile

import numpy as np


def main(argv=None) -> None:
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--workload", default="marlim_like_96")
    ap.add_argument("--op", choices=["A", "lusgs", "aphi", "csr"], default="lusgs")
    ap.add_argument("--prec", type=int, choices=[32, 64], default=32)
    ap.add_argument("--nsys", type=int, default=16)
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=2)
    ap.add_argument("--freq", type=float, default=0.5)
    ap.add_argument("--schedule", choices=["pipelined", "diagonal"], default="pipelined")
    ap.add_argument("--vw", type=int, default=0)
    ap.add_argument("--lines", type=int, default=1, help="lines per CTA of the complex64 pipelined sweeps")
    ap.add_argument("--systems", type=int, default=1,
                    help="systems of one frequency per CTA of the complex64 pipelined sweeps (1, 2, 4)")
    ap.add_argument("--split", type=int, default=1,
                    help="complex64 LU-SGS as a coalesced (B, w) pass and a light row pipeline (1, the "
                         "default) or one pass (0)")
    ap.add_argument("--overlap", type=int, default=1, help="split sweeps on two streams (1, the default) or one (0)")
    ap.add_argument("--cap", type=int, default=0, help="CTAs per SM of the split pipelines on two streams (0: none)")
    ap.add_argument("--by", type=int, default=8, help="stencil output rows per CTA")
    ap.add_argument("--ctas", type=int, default=4, help="stencil CTAs per SM of the plane chunks")
    ap.add_argument("--tiled", type=int, default=0, help="1: line-tiled complex64 LU-SGS sweeps")
    ap.add_argument("--tile-rows", type=int, default=8)
    ap.add_argument("--tile-vw", type=int, default=4)
    ap.add_argument("--check", action="store_true",
                    help="also apply the operator with the default schedule and report the difference")
    a = ap.parse_args(argv)

    import torch
    from . import api, synthetic
    cfg = synthetic.workload(a.workload)
    if a.op == "csr":
        cfg.params["airbc"] = 0
    airbc = int(cfg.params.get("airbc", 0))
    with tempfile.TemporaryDirectory() as d:
        G = synthetic.build_grid(cfg, d)
    ctx = api.Ctx(G, airbc, 0)
    if a.op == "csr":
        r = ctx.csr_compare(api.iom_of(a.freq), a.prec, a.reps)
        st_bytes = (2 * (16 if a.prec == 64 else 8) + (8 if a.prec == 64 else 4)) * ctx.lE
        r.update(workload=a.workload, airbc=0, prec=a.prec, unknowns=ctx.lE,
                 csr_GBps=r["csr_bytes"] / (r["ms_csr"] * 1e-3) / 1e9,
                 stencil_algorithmic_bytes=st_bytes,
                 stencil_GBps=st_bytes / (r["ms_stencil"] * 1e-3) / 1e9,
                 csr_over_stencil_time=r["ms_csr"] / r["ms_stencil"])
        print(json.dumps(r), flush=True)
        return
    ctx.set_option("lusgs_pipelined", 1 if a.schedule == "pipelined" else 0)
    ctx.set_option("lusgs_vw", a.vw)
    ctx.set_option("lusgs_lines", a.lines)
    ctx.set_option("lusgs_systems", a.systems)
    ctx.set_option("lusgs_split", a.split)
    ctx.set_option("lusgs_overlap", a.overlap)
    ctx.set_option("lusgs_cap", a.cap)
    ctx.set_option("stencil_by", a.by)
    ctx.set_option("stencil_ctas", a.ctas)
    ctx.set_option("lusgs_tiled", a.tiled)
    ctx.set_option("lusgs_tile_rows", a.tile_rows)
    ctx.set_option("lusgs_tile_vw", a.tile_vw)
    dt = torch.complex64 if a.prec == 32 else torch.complex128
    gen = torch.Generator(device="cuda").manual_seed(7)
    x = torch.randn(a.nsys, ctx.lE, dtype=dt, device="cuda", generator=gen)
    y = torch.empty_like(x)
    iom = np.zeros(2 * a.nsys)
    iom[1::2] = api.iom_of(a.freq).imag
    fn = {"A": api.lib().csem_fdfd_apply_dev, "lusgs": api.lib().csem_lusgs_apply_dev,
          "aphi": api.lib().csem_aphi_apply_dev}[a.op]
    torch.cuda.synchronize()
    stream = torch.cuda.ExternalStream(ctx.stream)

    def apply():
        rc = fn(ctx.h, a.prec, a.nsys, iom.ctypes.data_as(C.POINTER(C.c_double)), C.c_void_p(x.data_ptr()),
                C.c_void_p(y.data_ptr()), None)
        if rc:
            raise api.CsemError(rc, api.lib().csem_last_error().decode())

    for _ in range(a.warmup):
        apply()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(a.reps):
        apply()
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / a.reps
    nf = (ctx.n1 * (ctx.n2 + 1) * (ctx.n3f + 1) + (ctx.n1 + 1) * ctx.n2 * (ctx.n3f + 1)
          + (ctx.n1 + 1) * (ctx.n2 + 1) * ctx.n3f)
    bc = 16 if a.prec == 64 else 8
    bs = bc // 2
    per_sys = {"A": (2 * bc + bs) * ctx.lE, "lusgs": (5 * bc + 2 * bs) * nf, "aphi": None}[a.op]
    check = None
    if a.check:
        y1 = y.clone()
        ctx.set_option("lusgs_tiled", 0)
        ctx.set_option("lusgs_pipelined", 1)
        ctx.set_option("lusgs_vw", 0)
        ctx.set_option("lusgs_lines", 1)
        ctx.set_option("lusgs_systems", 1)
        ctx.set_option("lusgs_split", 0)
        apply()
        torch.cuda.synchronize()
        d = (y1 - y).abs().max().item()
        check = {"max_abs_diff": d, "rel": d / max(y.abs().max().item(), 1e-300),
                 "bit_identical": bool(torch.equal(torch.view_as_real(y1), torch.view_as_real(y)))}
    out = {"workload": a.workload, "op": a.op, "prec": a.prec, "nsys": a.nsys, "schedule": a.schedule,
           "vw": a.vw, "lines": a.lines, "systems": a.systems, "split": a.split, "overlap": a.overlap, "cap": a.cap, "by": a.by, "ctas": a.ctas, "tiled": a.tiled, "tile_rows": a.tile_rows, "tile_vw": a.tile_vw, "check": check,
           "ms_per_application": ms, "ms_per_system": ms / a.nsys,
           "algorithmic_bytes_per_system": per_sys,
           "algorithmic_GBps": per_sys * a.nsys / (ms * 1e-3) / 1e9 if per_sys else None}
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
