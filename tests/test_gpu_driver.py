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
        if f not in ("golden.npz", "args.json"):
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
