"""Host logic of the U(1) bond expansions (no GPU): the per-sector sketch of SketchedExpand
(sample_space / sketch_space, changebonds/randexpand.jl:160-165, sketchedexpand.jl:61-66)
draws exactly as the oracle's, the complement dimensions per charge, and the per-sector
selection of an oversampled sketch (truncspace(Vk))."""
import numpy as np
import pytest

from mpsgb import algorithms as A
from oracle import mps as P


@pytest.mark.parametrize("add,ov", [(3, 0), (5, 2), (40, 1)])
def test_u1_sketch_draws_like_the_oracle_and_respects_the_caps(add, ov):
    comp = {-2: 3, 0: 6, 2: 4, 4: 1}
    other = {-2: 1, 0: 5, 2: 7}
    dev, ora = A.SketchedExpand(add, ov, seed=11), P.SketchedExpand(add, ov, seed=11)
    for _ in range(3):
        qs, lc, kc = dev.sketch_u1(comp, other)
        oq, olc, okc = ora.sketch_u1(comp, other)
        assert qs.tolist() == oq.tolist() == [-2, 0, 2]
        assert lc.tolist() == olc.tolist() and kc.tolist() == okc.tolist()
        cap = np.array([1, 5, 4])
        assert kc.sum() == min(add, cap.sum())
        assert np.all(kc <= lc) and np.all(lc <= cap) and np.all(lc <= kc + ov)
        # the Gaussian draws that follow stay in step too
        assert np.array_equal(dev.gaussian(3, 2, np.float64), ora.gaussian(3, 2, np.float64))


def test_complement_dimensions_per_charge():
    q_fused = [-1, 1, 1, 3, 1, -1]
    q_bond = [-1, 1, 1]
    assert A._complement_dims(q_fused, q_bond) == {-1: 1, 1: 1, 3: 1}
    assert A._complement_dims(q_fused, q_fused) == {}
    assert P._u1_comp(q_fused, q_bond) == {-1: 1, 1: 1, 3: 1}


def test_sector_selection_keeps_the_leading_directions_of_each_sector(monkeypatch):
    captured = {}

    def fake_from_numpy(ctx, kind, arr, dtype=None):
        captured["S"] = np.asarray(arr)
        return "handle"
    monkeypatch.setattr(A.DeviceTensor, "from_numpy", staticmethod(fake_from_numpy))
    q = np.array([-2, -2, 0, 0, 0, 2, 2])
    sel, qk = A._sector_select(q, np.array([-2, 0, 2], np.int32), np.array([1, 2, 0]),
                               np.float64, None)
    S = captured["S"]
    assert sel == "handle" and qk.tolist() == [-2, 0, 0]
    assert S.shape == (3, 7) and S.sum() == 3
    assert [int(np.argmax(r)) for r in S] == [0, 2, 3]
    assert P._u1_keep(q, np.array([-2, 0, 2]), np.array([1, 2, 0])).tolist() == [0, 2, 3]
