"""Host logic of bench.py on CPU: the roofline arithmetic, the committed traffic figures it
reads, and the waves the default configuration walks."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def test_measured_traffic_reads_committed_profiles():
    import bench
    lus = bench.measured_traffic("lusgs32")
    st = bench.measured_traffic("stencil32")
    assert isinstance(lus, int) and isinstance(st, int)
    # the captures' DRAM bytes per system are of the order of the algorithmic bytes
    assert 0.5 < lus / (48 * 11911680) < 3.0
    assert 0.5 < st / (20 * 11064870) < 3.0
    assert bench.measured_traffic("A64") is None


def test_roofline_arithmetic():
    import bench
    res = {"lE": 11064870, "n1": 200, "n2": 140, "n3f": 140,
           # operator: (summed ms, applications, system-applications)
           "prof": {"stencil32": (1000.0, 100, 1600), "lusgs32": (7000.0, 100, 1600)}}
    dom, out = bench.roofline(res, {"hbm_gbs": 6689.5})
    assert dom == "lusgs32"
    nf = 200 * 141 * 141 + 201 * 140 * 141 + 201 * 141 * 140
    r = out["lusgs32"]
    assert r["algorithmic_bytes_per_system"] == 48 * nf
    # 16 systems per application, 70 ms per application
    assert r["achieved"] == pytest.approx(48 * nf * 16 / 0.070 / 1e9, abs=0.1)
    assert r["frac"] == pytest.approx(r["achieved"] / 6689.5, abs=1e-3)
    assert r["traffic"] == round(bench.measured_traffic("lusgs32") * 16)
    assert out["stencil32"]["achieved"] == pytest.approx(20 * 11064870 * 16 / 0.010 / 1e9, abs=0.1)
    # another grid: no captured traffic applies
    res["lE"] = 123
    assert bench.roofline(res, {})[1]["lusgs32"]["traffic"] is None


def test_default_waves_cover_the_batch_once(csem_lib):
    import bench
    from demo_matrixfree_csem_gb300 import synthetic
    cfg = synthetic.workload("marlim_like_96")  # the model in memory; nothing written
    freqs = [float(f) for f in cfg.params["freqs"].split(",")]
    systems = [(f, s) for f in freqs for s in range(len(cfg.acq.src))]
    assert len(systems) == 96 and len(freqs) == 6
    mine = bench.rank_systems(systems, 1, 0, 11064870)
    assert [(f, s) for f, s, r in mine] == systems  # one rank: the workload in its own order
    seen = []
    for k in range(2):  # the default: 2 timed steps of 48
        f, src = bench.wave_systems(cfg, mine, 48, k)
        assert len(f) == 48 and src.shape == (48, 3)
        seen += [(float(a), tuple(b)) for a, b in zip(f, src)]
    assert len(set(seen)) == 96


def test_reference_iteration_counts_come_from_the_reference_run():
    """The CPU legs extrapolate with the reference's own iteration counts on the bench
    model (its committed residual histories), not with published figures of another run."""
    import bench
    its = bench.reference_iterations("marlim_like_96")
    assert [its[f] for f in (0.125, 0.25, 0.5, 0.75, 1.0, 1.25)] == [1000, 1000, 641, 468, 391, 317]
    c128 = bench.complex128_iterations("marlim_like_96")
    assert len(c128) == 18 and all(v > 0 for v in c128)


def test_accuracy_field_flags_a_planted_error():
    """accuracy() compares the timed systems the complex128 fixture holds, per frequency
    and channel; an error planted in one receiver of one system shows up there and only
    there."""
    import bench
    from demo_matrixfree_csem_gb300 import synthetic
    z = np.load(os.path.join(bench.GOLDEN, "marlim_like_96", "fp64_receivers.npz"))
    cfg = synthetic.workload("marlim_like_96")
    dcal = {(round(float(z["freqs"][q]), 4), int(z["isrc"][q])): z["rec"][q].copy() for q in range(len(z["freqs"]))}
    a = bench.accuracy(cfg, dcal)
    assert a["systems"] == 18 and a["worst"] == 0.0
    key = (0.25, 7)
    r = int(np.argmax(np.abs(dcal[key][2])))
    dcal[key][2, r] *= 1 + 3e-6
    a = bench.accuracy(cfg, dcal)
    assert a["per_frequency"]["0.25"][2] > 1e-7 and a["per_frequency"]["0.25"][0] == 0.0
    assert all(max(v) == 0.0 for f, v in a["per_frequency"].items() if f != "0.25")


def test_wave_sources_follow_wave_systems(csem_lib):
    import bench
    from demo_matrixfree_csem_gb300 import synthetic
    cfg = synthetic.workload("marlim_like_96")
    freqs = [float(f) for f in cfg.params["freqs"].split(",")]
    systems = [(f, s) for f in freqs for s in range(len(cfg.acq.src))]
    mine = bench.rank_systems(systems, 2, 1, 11064870)
    for k in range(3):
        f, src = bench.wave_systems(cfg, mine, 48, k)
        idx = bench.wave_sources(mine, 48, k)
        want = cfg.acq.src[[i for i, _ in idx], :3].copy()
        want[:, 1] += 50.0 * np.array([r for _, r in idx], np.float32)
        assert np.array_equal(src, want)
