"""Throughput benchmark of the batched mixed-precision CSEM solve.

Workload (default): the 96-system Marlim-shaped batch - a seeded synthetic model of
180x120x120 core cells (200 m in x, 100 m in y,z) padded by nb=10 stretched cells to
200x140x140 (lextend=120 km), airwave boundary (airbc=1, 1024^2 FFT grid), 6 frequencies
(0.125-1.25 Hz) x 16 Ex sources = 96 systems, BiCGStab + LU-SGS, tol = 1e-8/f. The model
is generated by demo_matrixfree_csem_gb300.synthetic.marlim_like(seed=0).

A step solves one wave of `--wave` systems (default 48: the 16 sources at three
frequencies) to convergence, injection and receiver extraction included; steps walk the
96 systems in frequency order, so the 2 timed steps cover the whole batch once. Waves of
48 measured 7% more solves/s than waves of 16 (fewer steps in which only a few slow
systems keep the GPU busy); waves of all 96 a further 2%, at twice the time per step.

  value  solves/s with the model resident on the GPU, timed with CUDA events on the
         solver's stream over exactly K steps (synchronize + barrier on both sides);
  e2e    the same through the C ABI call a user makes (csem_solve_batch_host) with host
         (pinned) buffers for the per-step inputs (frequencies, source and receiver
         positions, channel lists) and outputs (receivers), timed on the host clock.

`--impl reference` times the reference's CPU implementation of the path instead (the
compiled reference when its sources are present, else the C restatement in oracle/) on
all host cores: one process per core, each timing a bounded number of iterations of one
system, extrapolated to whole solves with the reference's published Marlim iteration
counts (run_marlim/out.txt: 1000, 1000, 915, 696, 463, 354 iterations at 0.125-1.25 Hz).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

MARLIM_ITERS = {0.125: 1000, 0.25: 1000, 0.5: 915, 0.75: 696, 1.0: 463, 1.25: 354}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ----------------------------------------------------------------------------- workload
def make_workload(name: str, tmp: str):
    from demo_matrixfree_csem_gb300 import synthetic as syn
    try:
        cfg = syn.workload(name)
    except ValueError as e:
        raise SystemExit(str(e))
    syn.write_config(cfg, tmp)
    freqs = [float(f) for f in cfg.params["freqs"].split(",")]
    systems = [(f, s) for f in freqs for s in range(len(cfg.acq.src))]
    return cfg, freqs, systems


def grid_for(cfg, d):
    from demo_matrixfree_csem_gb300 import synthetic as syn
    return syn.build_grid(cfg, d)


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(gpu), f"--query-gpu={self.FIELDS}",
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self) -> dict:
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.count(",") >= 8]
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].strip() == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ----------------------------------------------------------------------------- CPU legs
def cpu_sample(workload: str, freq: float, iters: int, use_ref: bool) -> float:
    """Seconds per FBiCGStab+LU-SGS iteration of one system on one core."""
    code = f"""
import sys, time, os, numpy as np
sys.path.insert(0, {ROOT!r}); sys.path.insert(0, {os.path.join(ROOT, 'tests')!r})
import bench
cfg, freqs, systems = bench.make_workload({workload!r}, sys.argv[1])
d = sys.argv[1]
args = cfg.args(d)
if {use_ref!r}:
    from oracle import Ref
    R = Ref(args + ['niter={iters}'])
    ifreq = [float(f) for f in R.freqs].index(min(R.freqs, key=lambda f: abs(f - {freq})))
    x, b, t = R.solve(ifreq, niter={iters})
else:
    from cases import oracle_for, product_grid
    p = {{k: str(v) for k, v in cfg.params.items()}}
    G = product_grid(d, p)
    O = oracle_for(G, p)
    O.set_freq({freq})
    b = O.inject([0], cfg.acq.src[0])
    t0 = time.perf_counter()
    O.solve(b, algopt=1, precond=1, niter={iters}, tol=1e-30)
    t = time.perf_counter() - t0
print("SECONDS", t)
"""
    with tempfile.TemporaryDirectory() as d:
        r = subprocess.run([sys.executable, "-c", code, d], capture_output=True, text=True, cwd=ROOT)
    for line in r.stdout.splitlines():
        if line.startswith("SECONDS"):
            return float(line.split()[1]) / iters
    raise RuntimeError(f"CPU sample failed: {r.stderr[-2000:]}")


def cpu_baseline(workload: str, freqs, processes: int, iters: int):
    import oracle
    use_ref = oracle.ref_available() and os.path.exists(oracle.build_ref() or "")
    oracle.build_oracle()
    fmid = 0.5 if 0.5 in freqs else freqs[len(freqs) // 2]
    t0 = time.perf_counter()
    if processes == 1:
        spi = [cpu_sample(workload, fmid, iters, use_ref)]
    else:
        import concurrent.futures as cf
        with cf.ThreadPoolExecutor(processes) as ex:
            spi = list(ex.map(lambda _: cpu_sample(workload, fmid, iters, use_ref), range(processes)))
    wall = time.perf_counter() - t0
    s_it = statistics.mean(spi)
    its = statistics.mean(MARLIM_ITERS.get(round(f, 3), 700) for f in freqs)
    solves_per_s = processes / (s_it * its)
    return {"value": solves_per_s, "unit": "solves/s", "cores": processes,
            "kind": "reference" if use_ref else "port",
            "sample": (f"{processes} process(es) x {iters} FBiCGStab+LU-SGS iterations of one {workload} system at "
                       f"{fmid} Hz ({s_it:.3f} s/iteration, {wall:.1f} s wall); extrapolated with the reference's "
                       f"published Marlim iteration counts (mean {its:.0f} iterations per solve)")}


# ----------------------------------------------------------------------------- ranks
def wave_systems(cfg, systems, wave, k, rank):
    """Frequencies and source positions of step k on `rank`. Steps walk the system list
    in waves of `wave`; every rank owns its own sources (rank r's are shifted by 50 m * r
    along y), so the units of different ranks are disjoint and no data is exchanged
    (weak scaling)."""
    nwaves = (len(systems) + wave - 1) // wave
    w = k % nwaves
    sel = systems[w * wave:(w + 1) * wave]
    f = np.array([s[0] for s in sel], np.float32)
    src = np.stack([cfg.acq.src[s[1], :3] for s in sel]).astype(np.float32)
    src[:, 1] += 50.0 * rank
    return f, src


def max_over_ranks(values, device):
    """Element-wise maximum over all ranks of a list of floats (the timed region of the
    slowest rank)."""
    import torch
    import torch.distributed as tdist
    t = torch.tensor(values, dtype=torch.float64, device=device)
    tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
    return [float(v) for v in t]


# ----------------------------------------------------------------------------- FP64 drop-in leg
def fp64_dropin(ctx, cfg, freqs, iters: int):
    """The plain complex128 GPU drop-in (csem_solve_fp64_host: BiCGStab + LU-SGS, the
    reference's arithmetic) on one system of the workload: seconds per iteration from
    CUDA events on the solver's stream, extrapolated to whole solves with the same
    published Marlim iteration counts as the CPU legs."""
    import demo_matrixfree_csem_gb300 as cs
    import torch
    fmid = 0.5 if 0.5 in freqs else freqs[len(freqs) // 2]
    iom = cs.iom_of(fmid)
    b = ctx.inject_source(iom, ["Ex"], cfg.acq.src[0])
    st = torch.cuda.ExternalStream(ctx.stream)
    ctx.solve_fp64(iom, b, algopt=1, preco=1, niter=2, tol=1e-30)  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ctx.solve_fp64(iom, b, algopt=1, preco=1, niter=iters, tol=1e-30)
    torch.cuda.synchronize()
    s_it = (time.perf_counter() - t0) / iters
    its = statistics.mean(MARLIM_ITERS.get(round(f, 3), 700) for f in freqs)
    return {"value": 1.0 / (s_it * its), "unit": "solves/s", "s_per_iteration": s_it, "iterations_per_solve": its,
            "sample": (f"{iters} complex128 BiCGStab+LU-SGS iterations of one {cfg.name} system at {fmid} Hz through "
                       f"csem_solve_fp64_host (upload, solve, download); extrapolated with the reference's published "
                       f"Marlim iteration counts (mean {its:.0f} per solve)")}


# ----------------------------------------------------------------------------- GPU leg
def run_ours(args):
    import demo_matrixfree_csem_gb300 as cs
    import torch
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", 0))
    dist = world > 1
    if dist:
        import torch.distributed as tdist
        torch.cuda.set_device(local)
        tdist.init_process_group("nccl", device_id=torch.device("cuda", local))
    os.environ.setdefault("CUDA_VISIBLE_DEVICES", str(local))
    tmp = tempfile.mkdtemp()
    cfg, freqs, systems = make_workload(args.workload, tmp)
    G = grid_for(cfg, tmp)
    ctx = cs.Ctx(G, int(cfg.params["airbc"]), 0)
    rec = cfg.acq.rec
    wave = args.wave

    def step_systems(k):
        return wave_systems(cfg, systems, wave, k, rank)

    opts = dict(rec=rec, precision=32, preco=1, niter=args.niter, tol=1e-8, inner_tol=args.inner_tol,
                check_every=args.check_every, max_outer=args.max_outer)
    # pinned host staging for the e2e leg
    pin = {}

    def pinned(a):
        t = torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
        pin[id(t)] = t
        return t.numpy()

    log(f"[bench] {args.workload}: {len(systems)} systems, waves of {wave}, lE={ctx.lE}")
    for k in range(args.warmup):
        f, s = step_systems(k)
        cs.solve_batch(ctx, f, s, **opts)
    torch.cuda.synchronize()
    if dist:
        tdist.barrier()
    clocks = ClockSampler(local)
    cs.profile(True)
    l0 = cs.api.launch_count()
    nsolved = 0
    iters = []
    stat = []
    solver_stream = torch.cuda.ExternalStream(ctx.stream)  # the stream every solver kernel runs on
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    dev_ms = 0.0
    for k in range(args.warmup, args.warmup + args.steps):
        f, s = step_systems(k)
        fp, sp = pinned(f), pinned(s)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(solver_stream)
        r = cs.solve_batch(ctx, fp, sp, **opts)
        e1.record(solver_stream)
        e1.synchronize()
        dev_ms += e0.elapsed_time(e1)
        nsolved += len(f)
        iters += r["iters"].tolist()
        stat += r["status"]
    torch.cuda.synchronize()
    if dist:
        tdist.barrier()
    wall = time.perf_counter() - t0
    launches = cs.api.launch_count() - l0
    prof = cs.profile_read()
    cs.profile(False)
    ck = clocks.stop()
    if dist:
        wall, dev_s = max_over_ranks([wall, dev_ms / 1e3], "cuda")
        nsolved *= world
    else:
        dev_s = dev_ms / 1e3
    result = dict(wall=wall, dev_s=dev_s, nsolved=nsolved, iters=iters, status=stat, prof=prof, launches=launches,
                  clocks=ck, lE=ctx.lE, n1=ctx.n1, n2=ctx.n2, n3=ctx.n3, n3f=ctx.n3f, world=world, rank=rank)
    if args.fp64_iters > 0 and rank == 0:
        result["fp64"] = fp64_dropin(ctx, cfg, freqs, args.fp64_iters)
    return result, cfg, freqs, systems


def measured_traffic(kernel: str):
    """DRAM bytes per system and application of an operator from its committed ncu
    summary (the `traffic_bytes_per_system:` line), or None."""
    f = {"lusgs32": "k_sweep_lusgs32_marlim_like_96.md", "stencil32": "k_fdfd32_marlim_like_96.md"}.get(kernel)
    path = os.path.join(ROOT, "profiles", f) if f else None
    if not path or not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith("traffic_bytes_per_system:"):
            return int(line.split(":")[1])
    return None


def roofline(res, peaks):
    """Dominant operator (largest summed device time) and its algorithmic HBM bytes."""
    lE = res["lE"]
    nf = (res["n1"] * (res["n2"] + 1) * (res["n3f"] + 1) + (res["n1"] + 1) * res["n2"] * (res["n3f"] + 1)
          + (res["n1"] + 1) * (res["n2"] + 1) * res["n3f"])
    prof = res["prof"]
    # per-application algorithmic bytes of one system (complex64 inner operators):
    # stencil: read x and sigma, write y = (2*8 + 4) B per unknown;
    # LU-SGS: forward (read b, sigma; write y) + backward (read b, y, sigma; write y)
    #         = (5*8 + 2*4) B per unknown of the air-included grid
    bytes_per_sys = {"stencil32": 20 * lE, "lusgs32": 48 * nf}
    cands = {k: prof[k] for k in bytes_per_sys if prof[k][1] > 0}
    dom = max(cands, key=lambda k: cands[k][0])
    hbm = peaks.get("hbm_gbs", 6800.0)
    out = {}
    for k, (m, c, units) in cands.items():
        sys_per_app = units / c
        achieved = bytes_per_sys[k] * sys_per_app / (m / c / 1e3) / 1e9
        tps = measured_traffic(k) if res["lE"] == 11064870 else None  # captured on this workload only
        out[k] = {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm,
                  "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if "hbm_gbs" in peaks else "fallback",
                  "unit": "GB/s", "frac": round(achieved / hbm, 3),
                  "traffic": round(tps * sys_per_app) if tps else None,
                  "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of a 4-system capture, per "
                                    "system, times the systems per application" if tps else None,
                  "avg_ms": round(m / c, 4),
                  "applications": c, "systems_per_application": round(sys_per_app, 2),
                  "algorithmic_bytes_per_system": bytes_per_sys[k]}
    return dom, out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="marlim_like_96")
    ap.add_argument("--wave", type=int, default=48)
    ap.add_argument("--inner-tol", type=float, default=0.2)
    ap.add_argument("--check-every", type=int, default=4)
    ap.add_argument("--cpu-iters", type=int, default=3)
    ap.add_argument("--niter", type=int, default=1000,
                    help="inner iteration budget per system (the reference's niter); lower values are for "
                         "profiling runs, whose systems then stop unconverged")
    ap.add_argument("--max-outer", type=int, default=30, help="defect-correction cycles per system")
    ap.add_argument("--fp64-iters", type=int, default=8,
                    help="iterations of the complex128 drop-in timed for the fp64_dropin comparison (0: skip)")
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", 0))
    peaks = {}
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        peaks = json.load(open(pk))
    metric = "solves/s (batched mixed-precision CSEM solve, rel. residual < 1e-8/f)"
    tmp = tempfile.mkdtemp()
    if args.impl == "reference":
        if rank != 0:
            return
        cfg, freqs, systems = make_workload(args.workload, tmp)
        ncores = os.cpu_count() or 1
        # each step is one bounded sample on all cores; the line reports their mean
        samples = [cpu_baseline(args.workload, freqs, ncores, args.cpu_iters) for _ in range(max(1, args.steps))]
        cb = dict(samples[-1])
        cb["value"] = statistics.mean(x["value"] for x in samples)
        cb["sample"] = f"mean of {len(samples)} steps, each: " + cb["sample"]
        line = {"impl": "reference", "metric": metric, "value": cb["value"], "unit": "solves/s",
                "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": 1e3 * args.wave / cb["value"], "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "c128", "data": "synthetic",
                "config": {"workload": args.workload, "systems": len(systems), "wave": args.wave},
                "cpu_baseline": cb, "e2e": {"value": cb["value"], "unit": "solves/s", "h2d_bytes_per_step": 0,
                                            "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    res, cfg, freqs, systems = run_ours(args)
    if rank != 0:
        return
    value = res["nsolved"] / res["dev_s"]
    e2e = res["nsolved"] / res["wall"]
    dom, rf = roofline(res, peaks)
    nrec = len(cfg.acq.rec)
    h2d = args.wave * (4 + 12) + nrec * 20 + 4 + 12
    d2h = args.wave * 3 * nrec * 16
    line = {
        "metric": metric, "value": value, "unit": "solves/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * res["dev_s"] / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c64 inner / c128 outer", "data": "synthetic",
        "config": {"workload": args.workload, "systems": len(systems), "wave": args.wave, "grid": [res["n1"], res["n2"], res["n3"]],
                   "unknowns_per_system": res["lE"], "solver": "FBiCGStab+LU-SGS complex64 inner, complex128 defect correction",
                   "tol": "1e-8/f", "airbc": 1, "l2": "working set >> L2 (inputs larger than L2)",
                   "inner_tol": args.inner_tol},
        "roofline": rf[dom] | {"kernel": dom},
        "roofline_all": rf,
        "e2e": {"value": e2e, "unit": "solves/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": res["launches"],
        "clocks": res["clocks"],
        "iterations": {"mean_inner": float(np.mean(res["iters"])), "max_inner": int(np.max(res["iters"])),
                       "status": {s: res["status"].count(s) for s in set(res["status"])}},
        "operator_ms": {k: v for k, v in res["prof"].items() if v[1]},
    }
    if "fp64" in res:
        line["fp64_dropin"] = res["fp64"] | {"mixed_over_fp64": value / res["fp64"]["value"]}
    if not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(args.workload, freqs, 1, args.cpu_iters)
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
