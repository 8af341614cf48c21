"""The uneven-size batch: the bathymetry model (125x125x100 cells, Gaussian hills), the
96-system bench model (180x120x120 cells) and a 64^3 layered model, each padded with a
different nb per frequency (8 at 0.25 Hz, 10 at 0.75 Hz, 15 at 1.25 Hz), so the nine
contexts have nine grid sizes. All (model, frequency) batches run at the same time
through csem_solve_batches_host, complex64 GMRES(10) with LU-SGS inside complex128 defect
correction, to tol = 1e-8/f, and must:
  * converge, every system;
  * agree with the complex128 BiCGStab + LU-SGS solver (the reference's arithmetic) to
    1e-6 relative on the receivers, checked for one system per model at 1.25 Hz (both
    stop at the same true-residual level);
  * give exactly what a context gives when it runs alone.

The preconditioner is LU-SGS, not the reference's A-phi (fdfd.c:513-821). Its node sweeps
amplify a unit input to about 1e44 on the bathymetry model (complex128, measured), beyond
the complex64 range: the mixed path then stops the system with status "nonfinite", which
the last test checks. With the conductivity-weighted node diagonal (aphi_fix) A-phi stays
bounded, but GMRES(10) with it does not converge in a practical budget
(tests/test_gpu_aphi_fix.py)."""
import tempfile

import numpy as np
import pytest

import demo_matrixfree_csem_gb300 as cs
from demo_matrixfree_csem_gb300 import synthetic

pytestmark = pytest.mark.gpu

NB_OF_FREQ = {0.25: 8, 0.75: 10, 1.25: 15}
MODELS = {"bathymetry": (synthetic.bathymetry_125, 2), "bench": (lambda: synthetic.marlim_like(seed=0), 1),
          "layered64": (synthetic.layered_64, 1)}
OPTS = dict(algopt=2, nrestart=10, preco=1, niter=3000, tol=1e-8, max_outer=30)


@pytest.fixture(scope="module")
def jobs(gpu):
    out = []
    for name, (make, nsrc) in MODELS.items():
        for f, nb in NB_OF_FREQ.items():
            cfg = make()
            cfg.params["nb"] = nb
            with tempfile.TemporaryDirectory() as d:
                G = synthetic.build_grid(cfg, d)
            ctx = cs.Ctx(G, 1, 0)
            out.append(dict(name=name, cfg=cfg, job=dict(ctx=ctx, freqs=np.full(nsrc, f, np.float32),
                                                          srcs=cfg.acq.src[:nsrc, :3], rec=cfg.acq.rec, **OPTS)))
    return out


@pytest.fixture(scope="module")
def together(jobs):
    return cs.solve_batches([j["job"] for j in jobs])


def test_nine_grid_sizes(jobs):
    assert len({j["job"]["ctx"].lE for j in jobs}) == 9


def test_uneven_batch_converges_and_matches_complex128(jobs, together):
    for j, got in zip(jobs, together):
        assert got["status"] == ["converged"] * len(j["job"]["freqs"]), (j["name"], j["job"]["freqs"][0], got)
        print(f"{j['name']} {float(j['job']['freqs'][0])} Hz, {j['job']['ctx'].lE} unknowns: inner iterations "
              f"{got['iters'].tolist()}, defect corrections {got['outer'].tolist()}")
    for j, got in zip(jobs, together):
        if float(j["job"]["freqs"][0]) != 1.25:
            continue
        job = j["job"]
        r64 = cs.solve_batch(job["ctx"], job["freqs"][:1], job["srcs"][:1], rec=job["rec"], precision=64, algopt=1,
                             preco=1, niter=3000, tol=1e-8)
        assert r64["status"] == ["converged"]
        ref = r64["dcal"][0]
        err = float(np.abs(got["dcal"][0] - ref).max() / np.abs(ref).max())
        print(f"{j['name']} 1.25 Hz: mixed GMRES(10) vs complex128 BiCGStab {err:.2e}")
        assert err <= 1e-6, (j["name"], err)


def test_context_alone_matches_the_concurrent_batch(jobs, together):
    j, got = jobs[-1], together[-1]  # the 64^3 model, nb=15
    job = j["job"]
    args = {k: v for k, v in job.items() if k not in ("ctx", "freqs", "srcs")}
    alone = cs.solve_batch(job["ctx"], job["freqs"], job["srcs"], **args)
    assert np.array_equal(got["dcal"], alone["dcal"]) and got["status"] == alone["status"]


def test_aphi_overflow_is_reported(jobs):
    """The reference's A-phi on the bathymetry model: complex64 overflows and the system
    reports "nonfinite" (no NaN receivers are passed off as a result); complex128 stays
    finite."""
    job = jobs[0]["job"]
    args = dict(rec=job["rec"], algopt=2, nrestart=10, preco=3, niter=20, tol=1e-8, max_outer=1, inner_tol=1e-12)
    rng = np.random.default_rng(0)
    x = rng.standard_normal(job["ctx"].lE) + 1j * rng.standard_normal(job["ctx"].lE)
    y = job["ctx"].aphi_apply(cs.iom_of(0.25), x)
    assert np.all(np.isfinite(y)) and np.abs(y).max() > 1e38  # beyond the complex64 range
    r32 = cs.solve_batch(job["ctx"], job["freqs"][:2], job["srcs"][:2], precision=32, **args)
    assert r32["status"] == ["nonfinite"] * 2, r32["status"]
    r64 = cs.solve_batch(job["ctx"], job["freqs"][:1], job["srcs"][:1], precision=64, **args)
    assert np.all(np.isfinite(r64["dcal"]))
