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

  value     solves/s with the model resident on the GPU, timed with CUDA events on the
            solver's stream over exactly K steps (synchronize + barrier on both sides),
            with the product defaults (CUDA-graph replay of the inner iterations);
  e2e       the same through the C ABI call a user makes (csem_solve_batch_host) with
            host (pinned) buffers for the per-step inputs (frequencies, source and
            receiver positions, channel lists) and outputs (receivers), host clock;
  roofline  the dominant operator's algorithmic bytes per application over its average
            duration, from CUDA events around every application during one profiled
            wave (the last warm-up wave; profiling replaces graph replay by direct
            launches, so it is kept out of the timed steps);
  accuracy  max-norm relative receiver error per frequency and channel of the timed
            systems that tests/golden/marlim_like_96/fp64_receivers.npz also holds
            (complex128 solves of all six frequencies x sources 0, 7, 15).

`--impl reference` times the reference's CPU implementation of the path instead (the
compiled reference when its sources are present, else the C restatement in oracle/) on
all host cores: one process per core, each timing a bounded number of iterations of one
system; solves/s are extrapolated with the reference's own iteration counts on this
model (tests/golden/marlim_like_96/reference_receivers.npz: its BiCGStab + LU-SGS at
niter=1000 takes 1000, 1000, 641, 468, 391, 317 iterations at 0.125-1.25 Hz).
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

GOLDEN = os.path.join(ROOT, "tests", "golden")


def reference_iterations(workload: str) -> dict:
    """Iterations the reference itself takes per frequency on this workload (its
    residual history holds one entry per iteration plus the initial one while it
    converges, and exactly niter entries when it stops at niter)."""
    path = os.path.join(GOLDEN, workload, "reference_receivers.npz")
    z = np.load(path)
    out = {}
    for f in range(len(z["freqs"])):
        n = len(z[f"hist{f}"])
        out[round(float(z["freqs"][f]), 4)] = n if n >= 1000 else n - 1
    return out


def complex128_iterations(workload: str) -> list:
    """Iterations of the complex128 GPU solver on the systems of fp64_receivers.npz."""
    path = os.path.join(GOLDEN, workload, "fp64_receivers.npz")
    return [int(v) for v in np.load(path)["iters"]] if os.path.exists(path) else []


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
    from oracle.pyoracle import Oracle, setup_grid
    O = Oracle(setup_grid(d, {{k: str(v) for k, v in cfg.params.items()}}))
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
    """solves/s of the reference's CPU path on `processes` host cores: each process
    times `iters` FBiCGStab + LU-SGS iterations of one system of the workload; a whole
    solve takes the reference's own iteration count on this workload at each frequency."""
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
    ref_its = reference_iterations(workload)
    its = statistics.mean(ref_its[round(f, 4)] for f in freqs)
    solves_per_s = processes / (s_it * its)
    return {"value": solves_per_s, "unit": "solves/s", "cores": processes,
            "kind": "reference" if use_ref else "port",
            "sample": (f"{processes} process(es) x {iters} FBiCGStab+LU-SGS iterations of one {workload} system at "
                       f"{fmid} Hz ({s_it:.3f} s/iteration, {wall:.1f} s wall); a whole solve taken as the "
                       f"reference's own iteration count on this model (mean {its:.0f} over the frequencies: "
                       + "/".join(str(ref_its[round(f, 4)]) for f in freqs) + ")"),
            "sample_wall_s": wall, "seconds_per_iteration": s_it, "iterations_per_solve": its}


# ----------------------------------------------------------------------------- ranks
def rank_systems(systems, world, rank, unknowns):
    """The systems rank `rank` solves. Every rank owns a full copy of the workload
    (replica r has its sources shifted 50 m * r along y, so the units of different ranks
    are disjoint and no data is exchanged: weak scaling); the N copies are split over
    the ranks by the product's partitioner (csem_partition_systems: longest expected
    work first, work = unknowns * f^(-2/3)), then taken in frequency order. Entries are
    (frequency, source index, replica)."""
    import demo_matrixfree_csem_gb300 as cs
    allsys = [(f, s, r) for r in range(world) for (f, s) in systems]
    owner, _ = cs.partition_systems(world, [t[0] for t in allsys], unknowns=float(unknowns))
    mine = [t for t, o in zip(allsys, owner) if o == rank]
    return sorted(mine, key=lambda t: (t[0], t[2], t[1]))


def wave_systems(cfg, mine, wave, k):
    """Frequencies and source positions of step k: the rank's systems in waves of
    `wave`, cycling."""
    nwaves = (len(mine) + wave - 1) // wave
    w = k % nwaves
    sel = mine[w * wave:(w + 1) * wave]
    f = np.array([t[0] for t in sel], np.float32)
    src = np.stack([cfg.acq.src[t[1], :3] for t in sel]).astype(np.float32)
    src[:, 1] += 50.0 * np.array([t[2] for t in sel], np.float32)
    return f, src


def wave_sources(mine, wave, k):
    """(source index, replica) of the systems of step k, in wave order."""
    nwaves = (len(mine) + wave - 1) // wave
    w = k % nwaves
    return [(t[1], t[2]) for t in mine[w * wave:(w + 1) * wave]]


def max_over_ranks(values, device):
    """Element-wise maximum over all ranks of a list of floats (the timed region of the
    slowest rank)."""
    import torch
    import torch.distributed as tdist
    t = torch.tensor(values, dtype=torch.float64, device=device)
    tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
    return [float(v) for v in t]


# ----------------------------------------------------------------------------- FP64 drop-in leg
def fp64_dropin(ctx, cfg, freqs):
    """The plain complex128 GPU drop-in (csem_solve_fp64_host: BiCGStab + LU-SGS with the
    reference's arithmetic, one system at a time, as the reference's driver) on one whole
    system of the workload: source 0 at the highest frequency, solved to convergence and
    timed on the host around the call (upload, solve, download). Solves/s of the whole
    workload take that measured time per iteration and the complex128 solver's own
    iteration counts on the 18 systems of fp64_receivers.npz (all six frequencies)."""
    import demo_matrixfree_csem_gb300 as cs
    import torch
    f = max(freqs)
    iom = cs.iom_of(f)
    b = ctx.inject_source(iom, ["Ex"], cfg.acq.src[0])
    tol = float(np.float32(np.float32(1e-8) / np.float32(f)))
    ctx.solve_fp64(iom, b, algopt=1, preco=1, niter=2, tol=1e-30)  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    _, _, it, st = ctx.solve_fp64(iom, b, algopt=1, preco=1, niter=4000, tol=tol)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    s_it = wall / max(it, 1)
    its = complex128_iterations(cfg.name + "_96" if cfg.name == "marlim_like" else cfg.name)
    mean_its = statistics.mean(its) if its else float(it)
    return {"value": 1.0 / (s_it * mean_its), "unit": "solves/s", "s_per_iteration": s_it,
            "measured_solve": {"freq": f, "iterations": it, "status": st, "seconds": wall},
            "iterations_per_solve": mean_its,
            "sample": (f"one whole complex128 BiCGStab+LU-SGS solve of a {cfg.name} system at {f} Hz through "
                       f"csem_solve_fp64_host ({it} iterations, {wall:.1f} s); per solve the mean complex128 "
                       f"iteration count of {len(its)} systems at all six frequencies ({mean_its:.0f})")}


def accuracy(cfg, dcal_by_system):
    """Max-norm relative receiver error per frequency and channel against the complex128
    receivers of fp64_receivers.npz, over the timed systems that file holds."""
    path = os.path.join(GOLDEN, "marlim_like_96", "fp64_receivers.npz")
    if cfg.name != "marlim_like" or not os.path.exists(path):
        return None
    z = np.load(path)
    per = {}
    n = 0
    for q in range(len(z["freqs"])):
        key = (round(float(z["freqs"][q]), 4), int(z["isrc"][q]))
        if key not in dcal_by_system:
            continue
        got, ref = dcal_by_system[key], z["rec"][q]
        ex = np.abs(ref[0]).max()
        err = [float(np.abs(got[c] - ref[c]).max() / (np.abs(ref[c]).max() if c != 1 else ex)) for c in range(3)]
        f = str(key[0])
        per[f] = [max(a, b) for a, b in zip(per.get(f, [0.0] * 3), err)]
        n += 1
    if not n:
        return None
    return {"vs": "complex128 GPU solver (reference arithmetic, converged to 1e-8/f), "
                  "tests/golden/marlim_like_96/fp64_receivers.npz",
            "metric": "max-norm relative error over the receiver line; Ey against the Ex maximum",
            "channels": ["Ex", "Ey", "Ez"], "per_frequency": per, "systems": n,
            "worst": max(max(v) for v in per.values()), "target": 1e-7}


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

    mine = rank_systems(systems, world, rank, ctx.lE)

    def step_systems(k):
        return wave_systems(cfg, mine, wave, k)

    opts = dict(rec=rec, precision=32, preco=1, niter=args.niter, tol=1e-8, inner_tol=args.inner_tol,
                check_every=args.check_every, max_outer=args.max_outer)
    # pinned host staging for the e2e leg
    pin = {}

    def pinned(a):
        t = torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
        pin[id(t)] = t
        return t.numpy()

    for name, v in args.ctx_options.items():
        ctx.set_option(name, v)
    log(f"[bench] {args.workload}: {len(systems)} systems, waves of {wave}, lE={ctx.lE}")
    prof = None
    for k in range(args.warmup):
        f, s = step_systems(k)
        last = k == args.warmup - 1
        if last:  # per-operator CUDA events for the roofline, outside the timed steps
            cs.profile(True)
        cs.solve_batch(ctx, f, s, **opts)
        if last:
            torch.cuda.synchronize()
            prof = cs.profile_read()
            cs.profile(False)
    torch.cuda.synchronize()
    if dist:
        tdist.barrier()
    clocks = ClockSampler(local)
    l0 = cs.api.launch_count()
    nsolved = 0
    iters = []
    stat = []
    dcal = {}
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
        for q, (isrc, rep) in enumerate(wave_sources(mine, wave, k)):
            if rep == 0:  # the unshifted copy of the workload: comparable with the fixture
                dcal[(round(float(f[q]), 4), isrc)] = r["dcal"][q]
    torch.cuda.synchronize()
    if dist:
        tdist.barrier()
    wall = time.perf_counter() - t0
    launches = cs.api.launch_count() - l0
    ck = clocks.stop()
    if dist:
        wall, dev_s = max_over_ranks([wall, dev_ms / 1e3], "cuda")
        nsolved *= world
    else:
        dev_s = dev_ms / 1e3
    result = dict(wall=wall, dev_s=dev_s, nsolved=nsolved, iters=iters, status=stat, prof=prof, launches=launches,
                  clocks=ck, lE=ctx.lE, n1=ctx.n1, n2=ctx.n2, n3=ctx.n3, n3f=ctx.n3f, world=world, rank=rank,
                  accuracy=accuracy(cfg, dcal))
    if args.fp64 and rank == 0:
        result["fp64"] = fp64_dropin(ctx, cfg, freqs)
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
    ap.add_argument("--no-fp64", dest="fp64", action="store_false",
                    help="skip the whole complex128 drop-in solve of the fp64_dropin comparison")
    ap.add_argument("--ctx-option", action="append", default=[], metavar="NAME=VALUE",
                    help="a csem_ctx_set_option for the solver context (repeatable)")
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    args.ctx_options = {kv.split("=", 1)[0]: int(kv.split("=", 1)[1]) for kv in args.ctx_option}
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
        step_ms = 1e3 * statistics.mean(x["sample_wall_s"] for x in samples)
        line = {"impl": "reference", "metric": metric, "value": cb["value"], "unit": "solves/s",
                "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": step_ms, "ms_per_step_is": "wall time of one measured sample (all host cores)",
                "extrapolated_ms_per_wave": 1e3 * args.wave / cb["value"], "higher_is_better": True,
                "scaling": "weak",
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
                   "inner_tol": args.inner_tol, "options": args.ctx_options},
        "roofline": rf[dom] | {"kernel": dom},
        "roofline_all": rf,
        "roofline_source": "CUDA events on the solver stream around every operator application of the last "
                           "warm-up wave (direct launches); the timed steps replay CUDA graphs",
        "accuracy": res["accuracy"],
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
