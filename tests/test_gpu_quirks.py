"""The "fix_quirks" context option: source conductivity looked up at the source's own row.

With airbc=1 the reference shifts the source's full-grid row k by -nb before it reads
sigma11/sigma22 from the air-included model (inject_extract.c:55-63,81-89), so the
lookup lands nb rows too high, in the air for shallow sources. Parity mode (the default)
keeps that; fix_quirks=1 reads the rows k and k+1 of the source itself. Checks:
  * airbc=1, a source in the first Earth rows: b changes only at the source's Ex/Ey
    corners, and there by exactly the ratio of the two conductivities (to rounding);
    Ez (no conductivity) is bit-identical;
  * airbc=0 (no shift in the reference): the option changes nothing, bit for bit;
  * the option is per context and switches back.
"""
import numpy as np
import pytest

import demo_matrixfree_csem_gb300 as cs
from cases import product_grid
from demo_matrixfree_csem_gb300 import synthetic

pytestmark = pytest.mark.gpu


def _ctx(tmp_path, airbc):
    d = str(tmp_path)
    cfg = synthetic.random_small(77, nx=16, ny=14, nz=12, nb=4, airbc=airbc, n1fft=64, n2fft=64)
    synthetic.write_config(cfg, d)
    p = {k: str(v) for k, v in cfg.params.items()}
    G = product_grid(d, p)
    return cfg, G, cs.Ctx(G, airbc, 0)


def test_fix_quirks_source_sigma_row(gpu, tmp_path):
    cfg, G, ctx = _ctx(tmp_path, 1)
    A = G.arrays()
    n1, n2, n3f = G.shape_full
    nb = ctx.nb
    x3 = A["x3"]
    # a source in full-grid row nb+1: the reference's lookup reads rows 1 and 2 (air)
    z = 0.5 * (x3[nb + 1] + x3[nb + 2])
    src = np.array([cfg.acq.src[0][0], cfg.acq.src[0][1], z], np.float32)
    iom = cs.iom_of(0.5)
    b0 = ctx.inject_source(iom, ("Ex", "Ey", "Ez"), src)
    ctx.set_option("fix_quirks", 1)
    b1 = ctx.inject_source(iom, ("Ex", "Ey", "Ez"), src)
    ctx.set_option("fix_quirks", 0)
    b2 = ctx.inject_source(iom, ("Ex", "Ey", "Ez"), src)
    assert np.array_equal(b2.view(np.uint8), b0.view(np.uint8))  # switched back
    lEx, lEy = ctx.lEx, ctx.lEy
    assert np.array_equal(np.nonzero(b0)[0], np.nonzero(b1)[0])
    assert np.array_equal(b1[lEx + lEy:].view(np.uint8), b0[lEx + lEy:].view(np.uint8))  # Ez
    s11 = A["sigma11"].reshape(n3f + 1, n2 + 1, n1)
    s22 = A["sigma22"].reshape(n3f + 1, n2, n1 + 1)
    changed = 0
    for p in np.nonzero(b0[:lEx + lEy])[0]:
        if p < lEx:
            k, r = divmod(int(p), n1 * (n2 + 1))
            j, i = divmod(r, n1)
            sig_ref, sig_fix = s11[k, j, i], s11[k + nb, j, i]
        else:
            k, r = divmod(int(p) - lEx, (n1 + 1) * n2)
            j, i = divmod(r, n1 + 1)
            sig_ref, sig_fix = s22[k, j, i], s22[k + nb, j, i]
        want = sig_ref / sig_fix  # b ~ 1/sigma
        assert abs(b1[p] / b0[p] - want) <= 1e-13 * abs(want), (p, b1[p] / b0[p], want)
        changed += sig_ref != sig_fix
    assert changed > 0  # the reference's lookup did land in the air


def test_fix_quirks_no_effect_without_airbc(gpu, tmp_path):
    cfg, G, ctx = _ctx(tmp_path, 0)
    src = cfg.acq.src[0][:3]
    iom = cs.iom_of(1.0)
    b0 = ctx.inject_source(iom, ("Ex", "Ey", "Ez"), src)
    ctx.set_option("fix_quirks", 1)
    b1 = ctx.inject_source(iom, ("Ex", "Ey", "Ez"), src)
    assert np.array_equal(b1.view(np.uint8), b0.view(np.uint8))
