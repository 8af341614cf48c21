"""The uneven-size batch: the bathymetry model (125x125x100 cells, Gaussian hills) and a
64^3 layered model, each padded with a different nb per frequency (8, 10, 15), so the
six contexts have six grid sizes. All (model, frequency) batches run at the same time
through csem_solve_batches_host with complex64 GMRES(10) inside complex128 defect
correction, for a fixed budget, and must give exactly what each context gives alone.

The preconditioner is LU-SGS. The reference's A-phi preconditioner (fdfd.c:513-821)
amplifies a unit-size input to about 1e44 on the bathymetry model (measured in
complex128 at nb=8 and 15), which overflows complex64: the mixed path then stops the
system with status "nonfinite" and the complex128 path returns finite values, which the
last test checks."""
import tempfile

import numpy as np
import pytest

import demo_matrixfree_csem_gb300 as cs
from demo_matrixfree_csem_gb300 import synthetic

pytestmark = pytest.mark.gpu

NB_OF_FREQ = {0.25: 8, 0.75: 10, 1.25: 15}


@pytest.fixture(scope="module")
def jobs(gpu):
    out = []
    for cfg in (synthetic.bathymetry_125(), synthetic.layered_64()):
        for f, nb in NB_OF_FREQ.items():
            cfg.params["nb"] = nb
            with tempfile.TemporaryDirectory() as d:
                G = synthetic.build_grid(cfg, d)
            ctx = cs.Ctx(G, 1, 0)
            n = len(cfg.acq.src)
            out.append(dict(ctx=ctx, freqs=np.full(n, f, np.float32), srcs=cfg.acq.src[:, :3], rec=cfg.acq.rec,
                            algopt=2, nrestart=10, preco=1, niter=20, tol=1e-8, max_outer=1, inner_tol=1e-12))
    return out


def test_six_grid_sizes(jobs):
    sizes = {j["ctx"].lE for j in jobs}
    assert len(sizes) == 6


def test_concurrent_uneven_batch_matches_alone(jobs):
    together = cs.solve_batches(jobs)
    for j, got in zip(jobs, together):
        args = {k: v for k, v in j.items() if k not in ("ctx", "freqs", "srcs")}
        alone = cs.solve_batch(j["ctx"], j["freqs"], j["srcs"], **args)
        assert all(s in ("maxiter", "converged") for s in got["status"]), got["status"]
        assert np.all(np.isfinite(got["dcal"])) and np.all(got["relres"] < 1.0)
        assert np.array_equal(got["dcal"], alone["dcal"]) and got["status"] == alone["status"]


def test_aphi_overflow_is_reported(jobs):
    """A-phi on the bathymetry model: complex64 overflows and the system reports
    "nonfinite" (no NaN receivers are passed off as a result); complex128 stays finite."""
    j = jobs[0]
    args = dict(rec=j["rec"], algopt=2, nrestart=10, preco=3, niter=20, tol=1e-8, max_outer=1, inner_tol=1e-12)
    rng = np.random.default_rng(0)
    x = rng.standard_normal(j["ctx"].lE) + 1j * rng.standard_normal(j["ctx"].lE)
    y = j["ctx"].aphi_apply(cs.iom_of(0.25), x)
    assert np.all(np.isfinite(y)) and np.abs(y).max() > 1e38  # beyond the complex64 range
    r32 = cs.solve_batch(j["ctx"], j["freqs"][:2], j["srcs"][:2], precision=32, **args)
    assert r32["status"] == ["nonfinite"] * 2, r32["status"]
    r64 = cs.solve_batch(j["ctx"], j["freqs"][:1], j["srcs"][:1], precision=64, **args)
    assert np.all(np.isfinite(r64["dcal"]))
