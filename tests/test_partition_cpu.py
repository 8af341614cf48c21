"""The split of independent systems over devices (csem_partition_systems), on CPU.

Longest-work-first greedy over expected work unknowns x f^(-2/3) (or a given cost):
every system gets one slot, the split is deterministic, and the heaviest slot exceeds
the lightest by at most the largest single system's work (the greedy bound)."""
import numpy as np
import pytest


def _freqs96():
    return np.repeat(np.array([0.125, 0.25, 0.5, 0.75, 1.0, 1.25], np.float32), 16)


@pytest.mark.parametrize("ndev", [1, 2, 3, 4, 8])
def test_split_is_complete_balanced_and_deterministic(csem_lib, ndev):
    import demo_matrixfree_csem_gb300 as cs
    f = _freqs96()
    owner, load = cs.partition_systems(ndev, f, unknowns=11064870)
    assert owner.shape == (96,) and set(owner.tolist()) <= set(range(ndev))
    w = 11064870 * f.astype(np.float64) ** (-2.0 / 3.0)
    assert np.allclose([w[owner == d].sum() for d in range(ndev)], load)
    assert load.max() - load.min() <= w.max() * (1 + 1e-12)
    assert np.array_equal(owner, cs.partition_systems(ndev, f, unknowns=11064870)[0])
    if ndev <= 8:  # low frequencies are the heavy ones: no slot gets them all
        lows = [owner[f == 0.125].tolist().count(d) for d in range(ndev)]
        assert max(lows) - min(lows) <= 2 + 16 // ndev


def test_given_costs_and_errors(csem_lib):
    import demo_matrixfree_csem_gb300 as cs
    owner, load = cs.partition_systems(2, cost=[5.0, 4.0, 3.0, 3.0, 3.0])
    assert owner.tolist() == [0, 1, 1, 0, 1] and load.tolist() == [8.0, 10.0]
    with pytest.raises(cs.CsemError):
        cs.partition_systems(0, cost=[1.0])
    with pytest.raises(cs.CsemError):
        cs.partition_systems(2, cost=[1.0, -1.0])
    with pytest.raises(cs.CsemError):
        cs.partition_systems(2, freqs=[0.5, 0.0], unknowns=10)
    assert cs.partition_systems(3, cost=[])[0].shape == (0,)
