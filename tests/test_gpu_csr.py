"""The assembled operator (csem_csr_compare) against the matrix-free one.

A is assembled in CSR on the device by probing the stencil with 81 indicator vectors and
applied by cuSPARSE. On a golden case without the airwave (and on a larger random grid):
  * the SpMV and the stencil agree to rounding: <= 1e-13 relative in complex128 (the two
    sum the same products in different orders), <= 1e-5 in complex64;
  * 13 entries are stored per row;
  * a context with the airwave is refused (its top plane couples through an FFT), as the
    reference assembles A only without it (Acsr.c).
"""
import numpy as np
import pytest

import demo_matrixfree_csem_gb300 as cs
from cases import load_golden, parse_args, product_grid
from demo_matrixfree_csem_gb300 import synthetic

pytestmark = pytest.mark.gpu


def test_csr_matches_stencil_golden(gpu):
    d, args, gold = load_golden("lusgs_air0")
    p = parse_args(args)
    ctx = cs.Ctx(product_grid(d, p), 0, 0)
    iom = cs.iom_of(float(gold["freqs"][0]))
    r = ctx.csr_compare(iom, 64, 2)
    assert r["nnz"] == 13 * ctx.lE
    assert r["relerr"] <= 1e-13, r
    r32 = ctx.csr_compare(iom, 32, 2)
    assert r32["relerr"] <= 1e-5, r32


def test_csr_matches_stencil_multi_cta(gpu, tmp_path):
    cfg = synthetic.random_small(5, nx=40, ny=36, nz=30, nb=4, airbc=0)
    synthetic.write_config(cfg, str(tmp_path))
    ctx = cs.Ctx(product_grid(str(tmp_path), {k: str(v) for k, v in cfg.params.items()}), 0, 1)  # fvm=1
    r = ctx.csr_compare(cs.iom_of(0.75), 64, 2)
    assert r["relerr"] <= 1e-13, r


def test_csr_refuses_airwave(gpu):
    d, args, gold = load_golden("lusgs_air1")
    p = parse_args(args)
    ctx = cs.Ctx(product_grid(d, p), 1, 0)
    with pytest.raises(cs.CsemError):
        ctx.csr_compare(cs.iom_of(0.5), 64, 1)
