"""The FP64 adjoint in the oracle against FP64 central finite differences (CPU only).

This pins the hand-derived reverse of the step (the oracle's adjoint) before the CUDA adjoint
is compared with it."""
import numpy as np
import pytest

import oracle
from libcl_gb300 import params_derive
from libcl_gb300.scenes import SplitMix64, clone_params, differentiable_block

STEPS = 10


@pytest.fixture(scope="module")
def setup():
    sc = differentiable_block(8, 8, 8, seed=3)
    n = sc.n
    rng = SplitMix64(11)
    vel = np.zeros((n, 4))
    vel[:, :3] = rng.normal(3 * n).reshape(n, 3) * 0.1
    force = np.zeros((n, 4))
    force[:, :3] = np.array(list(sc.params.gravity)[:3])
    pos = sc.pos.astype(np.float64)
    tgt = pos.copy()
    tgt[:, :3] += 0.001 * rng.normal(3 * n).reshape(n, 3)
    return sc, pos, vel, force, tgt, rng


def _loss(sc, pos0, vel0, force, tgt, k=None, mu=None):
    P = clone_params(sc.params)
    if k is not None:
        P.stiffness = k
    if mu is not None:
        P.viscosity = mu
        params_derive(P)
    p, v, f = pos0.copy(), vel0.copy(), force.copy()
    oracle.run_f64(p, v, f, P, STEPS)
    return float(np.mean((p[:, :3] - tgt[:, :3]) ** 2)), p


def test_adjoint_f64_matches_central_differences(setup):
    sc, pos, vel, force, tgt, rng = setup
    n = sc.n
    _, pT = _loss(sc, pos, vel, force, tgt)
    gpos = np.zeros((n, 4))
    gpos[:, :3] = 2.0 * (pT[:, :3] - tgt[:, :3]) / (3 * n)
    gp0, gv0, gk, gmu = oracle.adjoint_f64(pos, vel, force, sc.params, STEPS, 4, gpos)
    eps = 1e-3
    k, mu = sc.params.stiffness, sc.params.viscosity
    fk = (_loss(sc, pos, vel, force, tgt, k=k + eps)[0] - _loss(sc, pos, vel, force, tgt, k=k - eps)[0]) / (2 * eps)
    fmu = (_loss(sc, pos, vel, force, tgt, mu=mu + eps)[0] - _loss(sc, pos, vel, force, tgt, mu=mu - eps)[0]) / (2 * eps)
    assert abs(gk - fk) <= 1e-3 * abs(fk), (gk, fk)
    assert abs(gmu - fmu) <= 1e-3 * abs(fmu), (gmu, fmu)
    for _ in range(4):
        d = np.zeros((n, 4))
        d[:, :3] = rng.normal(3 * n).reshape(n, 3)
        e = 1e-4
        fd = (_loss(sc, pos, vel + e * d, force, tgt)[0] - _loss(sc, pos, vel - e * d, force, tgt)[0]) / (2 * e)
        assert abs(np.sum(gv0 * d) - fd) <= 1e-6 * abs(fd), (np.sum(gv0 * d), fd)
        e = 1e-8  # positions: small enough not to switch a wall or a neighbour on or off
        fd = (_loss(sc, pos + e * d, vel, force, tgt)[0] - _loss(sc, pos - e * d, vel, force, tgt)[0]) / (2 * e)
        assert abs(np.sum(gp0 * d) - fd) <= 1e-4 * abs(fd), (np.sum(gp0 * d), fd)


def test_adjoint_f64_checkpoint_interval_is_invisible(setup):
    sc, pos, vel, force, tgt, rng = setup
    n = sc.n
    gpos = np.zeros((n, 4))
    gpos[:, :3] = rng.normal(3 * n).reshape(n, 3)
    gvel = np.zeros((n, 4))
    gvel[:, :3] = rng.normal(3 * n).reshape(n, 3)
    a = oracle.adjoint_f64(pos, vel, force, sc.params, STEPS, 3, gpos, gvel)
    b = oracle.adjoint_f64(pos, vel, force, sc.params, STEPS, STEPS, gpos, gvel)
    for x, y in zip(a[:2], b[:2]):
        np.testing.assert_array_equal(x, y)
    assert a[2] == b[2] and a[3] == b[3]


def test_adjoint_along_given_states_matches(setup):
    """The trajectory-driven FP64 adjoint, fed the FP64 run's own states rounded to FP32,
    agrees with the checkpointed FP64 adjoint to the size of that rounding."""
    sc, pos, vel, force, tgt, rng = setup
    n = sc.n
    p, v, f = pos.copy(), vel.copy(), force.copy()
    sp, sv = [], []
    for _ in range(STEPS):
        sp.append(p.astype(np.float32))
        sv.append(v.astype(np.float32))
        oracle.run_f64(p, v, f, sc.params, 1)
    gpos = np.zeros((n, 4))
    gpos[:, :3] = 2.0 * (p[:, :3] - tgt[:, :3]) / (3 * n)
    a = oracle.adjoint_f64(pos, vel, force, sc.params, STEPS, 4, gpos)
    b = oracle.adjoint_states_f64(np.stack(sp), np.stack(sv), force, sc.params, gpos)
    for x, y in zip(a[:2], b[:2]):
        assert np.linalg.norm(x - y) <= 1e-5 * np.linalg.norm(x)
    assert abs(a[2] - b[2]) <= 1e-5 * abs(a[2]) and abs(a[3] - b[3]) <= 1e-5 * abs(a[3])
