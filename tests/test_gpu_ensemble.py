"""Batched uneven BVE ensemble on the GPU: grouped launches, graph replay
and autotuning must reproduce the per-group RK4 kernels bitwise, and the
FP64 groups must match the oracle.  Tolerance: exact equality against the
per-group path (same per-member arithmetic), 1e-12 relative L2 against the
oracle, split-precision groups within 1e-10 of the FP64 groups."""
import numpy as np
import pytest
import torch

import oracle
from oracle import models as omodels
from helpers import rel_l2

import aeolus_gb300 as ae
from aeolus_gb300 import _lib, workloads as W
from aeolus_gb300.barotropic import BarotropicVorticity
from aeolus_gb300.ensemble import BarotropicEnsemble

pytestmark = pytest.mark.gpu
DEV = "cuda"
GROUPS = [(21, 32, 64, 3), (42, 64, 128, 2), (31, 48, 96, 4)]   # (l_max, nlat, nlon, members)


def _models(precision="fp64", nu=1e5, groups=None):
    ms = []
    for L, nlat, nlon, _ in groups or GROUPS:
        planet = ae.make_planet("latlon", nlat=nlat, nlon=nlon, l_max=L)
        if precision == "split":
            planet.so._product_space.sh.plan.set_precision(_lib.PREC_SPLIT_BF16)
        ms.append(BarotropicVorticity(planet, viscosity=nu))
    return ms


def _states(seed=0, groups=None):
    out = []
    for g, (L, _, _, B) in enumerate(groups or GROUPS):
        out.append(torch.as_tensor(np.stack([W.bve_vorticity(L, seed + 100 * g + b) for b in range(B)]), device=DEV))
    return out


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_grouped_step_equals_per_group_rk4(precision):
    models = _models(precision)
    ens = BarotropicEnsemble(models, [g[3] for g in GROUPS])
    states = _states()
    ref = [m.rk4(s.clone(), 900.0, 2) for m, s in zip(models, states)]
    ens.rk4(states, 900.0, 2)
    for a, b in zip(states, ref):
        assert torch.equal(a, b)


def test_fp64_groups_match_oracle():
    models = _models()
    ens = BarotropicEnsemble(models, [g[3] for g in GROUPS])
    states = _states(7)
    z0 = [s.cpu().numpy() for s in states]
    ens.rk4(states, 900.0, 1)
    for (L, nlat, nlon, B), s, z in zip(GROUPS, states, z0):
        sh = oracle.GaussSH(nlat, nlon, L)
        nf, mf = oracle.fine_dims(nlat, nlon, L)
        ops = oracle.Operators(sh, W.EARTH_RADIUS, sh_p=sh if (nf, mf) == (nlat, nlon) else oracle.GaussSH(nf, mf, L))
        for b in range(B):
            ref = omodels.bve_rk4_step(ops, z[b], 900.0, W.EARTH_OMEGA, 1e5)
            assert rel_l2(s[b].cpu().numpy(), ref) < 1e-12


def test_split_groups_close_to_fp64():
    a, b = _states(3), _states(3)
    BarotropicEnsemble(_models("split"), [g[3] for g in GROUPS]).rk4(a, 900.0, 4)
    BarotropicEnsemble(_models("fp64"), [g[3] for g in GROUPS]).rk4(b, 900.0, 4)
    for x, y in zip(a, b):
        assert rel_l2(x.cpu().numpy(), y.cpu().numpy()) < 1e-10


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_graph_replay_and_autotune_are_bitwise_neutral(precision):
    models = _models(precision)
    ens = BarotropicEnsemble(models, [g[3] for g in GROUPS])
    direct = _states(5)
    ens.rk4(direct, 600.0, 3)
    report = ens.autotune(_states(5))
    assert "row stage" in report
    tuned = _states(5)
    ens.rk4(tuned, 600.0, 3)
    graph = _states(5)
    ens.capture(graph, 600.0)
    ens.replay(3)
    torch.cuda.synchronize()
    for a, b, c in zip(direct, tuned, graph):
        assert torch.equal(a, b) and torch.equal(a, c)


def test_ensemble_rejects_bad_input():
    models = _models()
    with pytest.raises(ValueError):
        BarotropicEnsemble(models, [1, 2])
    ens = BarotropicEnsemble(models, [g[3] for g in GROUPS])
    bad = _states()
    bad[1] = bad[1][:1].clone()
    with pytest.raises(ValueError):
        ens.rk4(bad, 600.0)
    with pytest.raises(RuntimeError):
        ens.replay(1)


# nlon 384 (prime-factor row body), 256 (fixed-radix row body) and 64
# (runtime-radix row body) in one grouped launch
FIXED_BODY_GROUPS = [(127, 192, 384, 2), (85, 128, 256, 2), (21, 32, 64, 2)]


def test_grouped_split_step_equals_per_group_rk4_on_every_row_body():
    models = _models("split", groups=FIXED_BODY_GROUPS)
    ens = BarotropicEnsemble(models, [g[3] for g in FIXED_BODY_GROUPS])
    states = _states(5, groups=FIXED_BODY_GROUPS)
    ref = [m.rk4(s.clone(), 900.0, 2) for m, s in zip(models, states)]
    ens.rk4(states, 900.0, 2)
    for a, b in zip(states, ref):
        assert torch.equal(a, b)
