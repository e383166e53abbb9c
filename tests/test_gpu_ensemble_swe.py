"""Batched uneven SWE ensemble on the GPU.  Split-precision groups reproduce
the per-group ShallowWaterModel.rk4 bitwise (integer and double-float
arithmetic with explicit error-free operations); FP64 groups agree to 1e-14
relative L2 per field -- the same FP64 expressions, inlined into the grouped
kernels of another translation unit, may be contracted into FMAs differently,
which moves the last bit of a few coefficients (measured: 1 ulp).  Graph
replay and autotuning are bitwise neutral; split groups stay within 1e-10 of
the FP64 groups (the stated accuracy of the split form)."""
import numpy as np
import pytest
import torch

from helpers import rel_l2

import aeolus_gb300 as ae
from aeolus_gb300 import _lib, workloads as W
from aeolus_gb300.ensemble import BarotropicEnsemble, ShallowWaterEnsemble
from aeolus_gb300.shallow_water import ShallowWaterModel

pytestmark = pytest.mark.gpu
DEV = "cuda"
GROUPS = [(21, 32, 64, 3), (42, 64, 128, 2), (31, 48, 96, 2)]   # (l_max, nlat, nlon, members)


def _models(precision="fp64", groups=None):
    ms, depths = [], []
    for g, (L, nlat, nlon, B) in enumerate(groups or GROUPS):
        planet = ae.make_planet("latlon", nlat=nlat, nlon=nlon, l_max=L)
        if precision == "split":
            planet.so._product_space.sh.plan.set_precision(_lib.PREC_SPLIT_BF16)
        _, depth = W.member_states(L, B, seed=11 + g)
        ms.append(ShallowWaterModel(planet, gravity=W.GRAVITY, mean_depth=depth))
    return ms


def _states(groups=None):
    return [torch.as_tensor(W.member_states(L, B, seed=11 + g)[0], device=DEV)
            for g, (L, _, _, B) in enumerate(groups or GROUPS)]


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_grouped_swe_step_equals_per_group_rk4(precision):
    models = _models(precision)
    ens = ShallowWaterEnsemble(models, [g[3] for g in GROUPS])
    states = _states()
    ref = [m.rk4(s.clone(), 300.0, 2, check=False) for m, s in zip(models, states)]
    ens.rk4(states, 300.0, 2)
    for a, b in zip(states, ref):
        if precision == "split":
            assert torch.equal(a, b)
        else:
            for f in range(3):
                assert rel_l2(a[:, f].cpu().numpy(), b[:, f].cpu().numpy()) < 1e-14


def test_split_swe_groups_close_to_fp64():
    a, b = _states(), _states()
    ShallowWaterEnsemble(_models("split"), [g[3] for g in GROUPS]).rk4(a, 300.0, 3)
    ShallowWaterEnsemble(_models("fp64"), [g[3] for g in GROUPS]).rk4(b, 300.0, 3)
    for x, y in zip(a, b):
        for f in range(3):
            assert rel_l2(x[:, f].cpu().numpy(), y[:, f].cpu().numpy()) < 1e-10


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_swe_graph_replay_and_autotune_are_bitwise_neutral(precision):
    models = _models(precision)
    ens = ShallowWaterEnsemble(models, [g[3] for g in GROUPS])
    direct = _states()
    ens.rk4(direct, 300.0, 2)
    assert "row stage" in ens.autotune(_states())
    tuned = _states()
    ens.rk4(tuned, 300.0, 2)
    graph = _states()
    ens.capture(graph, 300.0)
    ens.replay(2)
    torch.cuda.synchronize()
    for a, b, c in zip(direct, tuned, graph):
        assert torch.equal(a, b) and torch.equal(a, c)


def test_swe_ensemble_rejects_bad_input():
    models = _models()
    with pytest.raises(ValueError):
        ShallowWaterEnsemble(models, [1, 2])
    ens = ShallowWaterEnsemble(models, [g[3] for g in GROUPS])
    bad = _states()
    bad[0] = bad[0][:, :2].contiguous()
    with pytest.raises(ValueError):
        ens.rk4(bad, 300.0)
    # a BVE step on an SWE ensemble is refused by the library
    zeta = [s[:, 0].contiguous() for s in _states()]
    with pytest.raises(Exception):
        BarotropicEnsemble.rk4(ens, zeta, 300.0)


# nlon 384 (prime-factor row body), 256 (fixed-radix row body) and 64
# (runtime-radix row body) in one grouped launch
FIXED_BODY_GROUPS = [(127, 192, 384, 2), (85, 128, 256, 2), (21, 32, 64, 2)]


def test_grouped_split_swe_step_equals_per_group_rk4_on_every_row_body():
    models = _models("split", groups=FIXED_BODY_GROUPS)
    ens = ShallowWaterEnsemble(models, [g[3] for g in FIXED_BODY_GROUPS])
    states = _states(groups=FIXED_BODY_GROUPS)
    ref = [m.rk4(s.clone(), 300.0, 2, check=False) for m, s in zip(models, states)]
    ens.rk4(states, 300.0, 2)
    for a, b in zip(states, ref):
        assert torch.equal(a, b)
