"""The key=value driver `csem` against the reference's own output files.

For every golden case without the airwave, the driver runs the case's command line (the
reference's flags, float32 model files, sources.txt / receivers.txt) at the first
frequency with dot_order=1, i.e. the reference's summation order in the dot products.
The solve then repeats the reference's arithmetic, so the files the driver writes must
be the reference's text exactly:
  * emf_0001.txt: the header and one "%d \\t %d \\t %d \\t %d \\t %e \\t %e" row per channel
    and receiver (write_data.c:24-32), the values being the reference's complex64
    receivers of the fixture;
  * iterate_<solver>.txt: the residual history the reference printed, in its format.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

from cases import GOLDEN_CASES, load_golden, parse_args

pytestmark = pytest.mark.gpu

AIR0 = [c for c in GOLDEN_CASES if parse_args(load_golden(c)[1]).get("airbc", "0") == "0"]


def _hist_file(p):
    algopt, preco = int(p.get("algopt", 1)), int(p.get("preco", 1))
    if algopt == 1:
        return "iterate_fbicgstab.txt" if preco else "iterate_bicgstab.txt"
    return "iterate_fgmres.txt" if preco else "iterate_gmres.txt"


@pytest.mark.parametrize("case", AIR0)
def test_driver_writes_reference_files(gpu, case, tmp_path):
    from demo_matrixfree_csem_gb300 import build
    d, args, gold = load_golden(case)
    for f in os.listdir(d):
        if os.path.isfile(os.path.join(d, f)) and f not in ("golden.npz", "args.json"):
            shutil.copy(os.path.join(d, f), tmp_path / f)
    p = parse_args(args)
    f0 = float(gold["freqs"][0])
    run = subprocess.run([build.DRIVER, *args[1:], f"freqs={p['freqs'].split(',')[0]}", "dot_order=1", "verb=1"],
                         cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert run.returncode == 0, run.stderr
    assert abs(f0 - float(p["freqs"].split(",")[0])) < 1e-6
    emf = open(tmp_path / "emf_0001.txt").read()
    dcal = gold["dcal"]  # [nchrec][nrec] complex64 at the first frequency
    rows = ["iTx \t iRx    ichrec  ifreq \t emf_real \t emf_imag\n"]
    for c in range(dcal.shape[0]):
        for r in range(dcal.shape[1]):
            v = dcal[c, r]
            rows.append("%d \t %d \t %d \t %d \t %e \t %e\n" % (1, r + 1, c + 1, 1, float(v.real), float(v.imag)))
    assert emf == "".join(rows)
    hist = open(tmp_path / _hist_file(p)).read().splitlines()
    printed = gold["hist_printed"]
    assert len(hist) == len(printed) + 1
    assert [float(ln.split()[1]) for ln in hist[1:]] == [float("%e" % v) for v in printed]


def test_driver_all_sources_writes_one_file_per_source(gpu, tmp_path):
    """nsrc=all solves every source row (the reference solves only the first,
    acq_init_free.c:56,90) and writes emf_0001.txt, emf_0002.txt, ... in the
    write_data.c:24-32 format, source s with iTx = s. Each file equals what the driver
    writes for that source alone (iTx aside), and the batched mixed-precision driver
    (precision=32) gives the same receivers to complex64 output precision."""
    from demo_matrixfree_csem_gb300 import build
    case = "lusgs_air0"
    d, args, gold = load_golden(case)
    for f in os.listdir(d):
        if os.path.isfile(os.path.join(d, f)) and f not in ("golden.npz", "args.json", "acsr.npz"):
            shutil.copy(os.path.join(d, f), tmp_path / f)
    lines = open(tmp_path / "sources.txt").read().splitlines()
    head, row = lines[0], lines[1].split()
    srcs = []
    for s, dx in enumerate((0.0, 45.0, -60.0)):
        r = list(row)
        r[0] = "%f" % (float(row[0]) + dx)
        r[5] = str(s + 1)
        srcs.append(" ".join(r))
        (tmp_path / f"one_{s + 1}.txt").write_text(head + "\n" + " ".join(r[:5] + ["1"]) + "\n")
    (tmp_path / "three.txt").write_text(head + "\n" + "\n".join(srcs) + "\n")
    base = [a for a in args[1:] if not a.startswith("fsrc=")] + ["niter=400"]

    def run(extra, cwd):
        r = subprocess.run([build.DRIVER, *base, *extra], cwd=cwd, capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr
        return r

    all_dir = tmp_path / "all"
    all_dir.mkdir()
    for f in os.listdir(tmp_path):
        if os.path.isfile(tmp_path / f):
            shutil.copy(tmp_path / f, all_dir / f)
    run(["fsrc=three.txt", "nsrc=all"], all_dir)
    p = parse_args(args)
    nfreq, nch = len(p["freqs"].split(",")), len(p["chrec"].split(","))
    for s in range(3):
        one = tmp_path / f"single_{s + 1}"
        one.mkdir()
        for f in os.listdir(tmp_path):
            if os.path.isfile(tmp_path / f):
                shutil.copy(tmp_path / f, one / f)
        run([f"fsrc=one_{s + 1}.txt"], one)
        got = open(all_dir / f"emf_{s + 1:04d}.txt").read().splitlines()
        want = open(one / "emf_0001.txt").read().splitlines()
        assert got[0] == want[0] == "iTx \t iRx    ichrec  ifreq \t emf_real \t emf_imag"
        assert len(got) == 1 + nch * nfreq * len(gold["dcal"][0])
        for g_, w_ in zip(got[1:], want[1:]):
            gf, wf = g_.split(" \t "), w_.split(" \t ")
            assert gf[0] == str(s + 1) and wf[0] == "1" and gf[1:] == wf[1:]
    assert not os.path.exists(all_dir / "emf_0004.txt")


def test_driver_all_sources_mixed_precision_matches_complex128(gpu, tmp_path):
    """The batched mixed-precision driver (precision=32: every (source, frequency) system
    in one batch) reports every system converged and writes, per source, the receivers
    of the complex128 driver to 1e-5 relative. On a 40 x 27 x 19 cell model with three
    sources and the airwave boundary (airbc=1), the setting of every mixed-precision
    workload: with airbc=0 the air layers are part of the operator and the complex64
    inner solves stagnate near a relative residual of 1e-7 (the mixed solver then
    reports maxiter; measured on this model and on the golden ones)."""
    from demo_matrixfree_csem_gb300 import build, synthetic
    cfg = synthetic.random_small(71, nx=40, ny=27, nz=19, nb=4, airbc=1, fvm=0, n1fft=64, n2fft=64)
    synthetic.write_config(cfg, str(tmp_path))
    lines = open(tmp_path / "sources.txt").read().splitlines()
    head, row = lines[0], lines[1].split()
    srcs = []
    for s, dx in enumerate((0.0, 150.0, -220.0)):
        r = list(row)
        r[0] = "%f" % (float(row[0]) + dx)
        r[5] = str(s + 1)
        srcs.append(" ".join(r))
    (tmp_path / "three.txt").write_text(head + "\n" + "\n".join(srcs) + "\n")
    base = [a for a in cfg.args(str(tmp_path))[1:] if not a.startswith("fsrc=")]
    base += [f"fsrc={tmp_path}/three.txt", "nsrc=all", "niter=1000"]
    out = {}
    for prec in (64, 32):
        d = tmp_path / f"p{prec}"
        d.mkdir()
        r = subprocess.run([build.DRIVER, *base, f"precision={prec}", "verb=1"], cwd=d, capture_output=True,
                           text=True, timeout=600)
        assert r.returncode == 0, r.stderr
        if prec == 32:
            st = [ln for ln in r.stdout.splitlines() if ln.startswith("source ") and "status" in ln]
            assert len(st) == 3 * len(cfg.params["freqs"].split(",")), st
            assert all("status 1," in ln for ln in st), st  # CSEM_ST_CONVERGED
        out[prec] = [np.array([[float(v) for v in ln.split(" \t ")[4:6]] for ln in
                               open(d / f"emf_{s + 1:04d}.txt").read().splitlines()[1:]]) for s in range(3)]
    for s in range(3):
        a, b = out[64][s], out[32][s]
        assert np.abs(a - b).max() <= 1e-5 * np.abs(a).max(), (s, np.abs(a - b).max() / np.abs(a).max())
