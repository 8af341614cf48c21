"""The same-symbol drop-in (libcsem_refabi.so) links with the reference's own driver.

Where the reference sources are present, its main.c and set-up/I-O files
(emf_init_free.c, acq_init_free.c, extend_model.c, create_nugrid.c, find_index.c,
write_data.c, cstd.c, Acsr.c) are compiled unmodified and linked against
libcsem_refabi.so instead of fdfd.c / airbc_init_free.c / inject_extract.c /
cdotprod.c / solver.c / gmres_init_free.c. The struct layouts the drop-in declares are
checked against the reference's emf.h / acq.h. Without a GPU the linked driver must
stop with the library's error message (exit status 1, as err()); with a GPU it must
reproduce the golden receivers.
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
from oracle.pyoracle import REF_SRC as REF  # noqa: E402
pytestmark = pytest.mark.skipif(not os.path.exists(os.path.join(REF, "main.c")),
                                reason="reference sources not present")

REF_FILES = ["main.c", "emf_init_free.c", "acq_init_free.c", "extend_model.c", "create_nugrid.c", "find_index.c",
             "write_data.c", "cstd.c", "Acsr.c"]


@pytest.fixture(scope="module")
def dropin(tmp_path_factory, csem_lib):
    from demo_matrixfree_csem_gb300 import build
    build.build()
    d = tmp_path_factory.mktemp("dropin")
    exe = str(d / "main_dropin")
    srcs = [os.path.join(REF, f) for f in REF_FILES] + [os.path.join(ROOT, "oracle", "ref_stubs", "ref_stubs.c"),
                                                      os.path.join(ROOT, "oracle", "fft2d.c")]
    cmd = ["gcc", "-O2", "-w", "-std=gnu99", "-I", os.path.join(ROOT, "oracle", "ref_stubs"), "-I", REF, *srcs,
           "-o", exe, f"-L{build.OUT}", "-lcsem_refabi", "-lcsem_gpu", f"-Wl,-rpath,{build.OUT}", "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe, d


def test_struct_layout_matches_reference(tmp_path, csem_lib):
    from demo_matrixfree_csem_gb300 import build
    build.build()
    probe = tmp_path / "probe.c"
    probe.write_text("""
#include <stdio.h>
#include <stddef.h>
#include "cstd.h"
#include "emf.h"
#include "acq.h"
int main(void) {
  printf("%ld %ld %ld %ld %ld %ld %ld %ld\\n", (long)sizeof(emf_t), (long)sizeof(acq_t),
         (long)offsetof(emf_t, sigma11), (long)offsetof(emf_t, I_omega_mu0), (long)offsetof(emf_t, dcal_fd),
         (long)offsetof(emf_t, param_extended), (long)offsetof(acq_t, rec_x1), (long)offsetof(acq_t, shot_idx));
  return 0;
}
""")
    exe = str(tmp_path / "probe")
    subprocess.run(["gcc", "-I", REF, str(probe), "-o", exe], check=True)
    ref = [int(v) for v in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()]
    lib = ctypes.CDLL(build.REFABI)
    out = (ctypes.c_long * 8)()
    lib.csem_refabi_layout(out)
    assert list(out) == ref


def test_reference_driver_links_and_runs(dropin):
    import demo_matrixfree_csem_gb300 as cs
    from cases import load_golden
    exe, d = dropin
    gdir, args, gold = load_golden("lusgs_air1")
    run = subprocess.run([exe, *args[1:], "verb=1"], cwd=gdir, capture_output=True, text=True, timeout=600)
    if cs.device_count() == 0:
        assert run.returncode == 1 and "no CUDA device available" in run.stderr
        return
    assert run.returncode == 0, run.stderr
    lines = open(os.path.join(gdir, "emf_0001.txt")).read().splitlines()[1:]
    vals = np.array([[float(v) for v in ln.split()[4:6]] for ln in lines])
    for f in ("emf_0001.txt", "iterate_fbicgstab.txt"):
        os.remove(os.path.join(gdir, f))
    nch, nrec = gold["dcal"].shape
    nf = len(gold["freqs"])
    got = vals.reshape(nch, nf, nrec, 2)[:, 0]          # rows: ichrec > ifreq > irec (write_data.c:26-28)
    want = np.stack([gold["dcal"].real, gold["dcal"].imag], axis=-1)
    np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-6 * np.abs(want).max())
