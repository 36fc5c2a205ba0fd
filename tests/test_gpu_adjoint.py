"""The CUDA adjoint of the 3D step (gbsph_adjoint3d_*) against the FP64 oracle adjoint and
central finite differences of the CUDA forward step.

Loss throughout: L = mean over particles and x, y, z of (x_T - target_T)^2 after T steps, the
target being the same simulator run from perturbed initial velocities with viscosity 0.08."""
import numpy as np
import pytest

from libcl_gb300 import ERR_ARGUMENT, ERR_STATE, KEY_REFERENCE_HASH, Adjoint3D, GbsphError, params_derive
from libcl_gb300.scenes import SplitMix64, clone_params, differentiable_block, perturbed_velocities

from fluid_helpers import make_fluid, set_params

pytestmark = pytest.mark.gpu

# gradients of the FP32 CUDA adjoint against the FP64 oracle adjoint: relative error of the
# velocity field (in the 2-norm) and of each parameter derivative
GRAD_RTOL = 1e-3


def gravity4(sc):
    f = np.zeros_like(sc.pos)
    f[:, :3] = np.array(list(sc.params.gravity)[:3], np.float32)
    return f


def target_positions(sc, steps):
    """Final positions of the target run: v0 + N(0, 0.1^2) (seed 6) and viscosity 0.08."""
    import torch
    p = clone_params(sc.params)
    p.viscosity = 0.08
    params_derive(p)
    f = make_fluid(sc, vel=perturbed_velocities(sc.vel), force=gravity4(sc))
    set_params(f, p)
    for _ in range(steps):
        f.compute()
    torch.cuda.synchronize()
    return f.getPositionBuffer().cpu().numpy().astype(np.float64)


def gpu_gradients(sc, steps, every, tgt, vel=None):
    import torch
    f = make_fluid(sc, vel=vel, force=gravity4(sc))
    adj = Adjoint3D(f, steps, every)
    adj.forward()
    pos = f.getPositionBuffer().clone()
    n = sc.n
    gpos = torch.zeros_like(pos)
    gpos[:, :3] = 2.0 * (pos[:, :3].double() - torch.from_numpy(tgt[:, :3]).cuda()).float() / (3 * n)
    gp0, gv0, gpar = adj.backward(gpos)
    torch.cuda.synchronize()
    loss = float(torch.mean((pos[:, :3].double() - torch.from_numpy(tgt[:, :3]).cuda()) ** 2))
    return dict(loss=loss, gp0=gp0.cpu().numpy(), gv0=gv0.cpu().numpy(), gk=float(gpar[0]), gmu=float(gpar[1]),
                pos=pos.cpu().numpy(), fluid=f, adj=adj)


def oracle_gradients(olib, sc, steps, every, tgt, vel=None):
    n = sc.n
    pos0 = sc.pos.astype(np.float64)
    vel0 = (sc.vel if vel is None else vel).astype(np.float64)
    force0 = gravity4(sc).astype(np.float64)
    p, v, fo = pos0.copy(), vel0.copy(), force0.copy()
    olib.run_f64(p, v, fo, sc.params, steps)
    gpos = np.zeros((n, 4))
    gpos[:, :3] = 2.0 * (p[:, :3] - tgt[:, :3]) / (3 * n)
    gp0, gv0, gk, gmu = olib.adjoint_f64(pos0, vel0, force0, sc.params, steps, every, gpos)
    return dict(gp0=gp0, gv0=gv0, gk=gk, gmu=gmu, pos=p)


def field_rel(a, b):
    a = np.asarray(a, np.float64)[:, :3]
    b = np.asarray(b, np.float64)[:, :3]
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def check_against_oracle(g, o):
    assert field_rel(g["gv0"], o["gv0"]) < GRAD_RTOL, field_rel(g["gv0"], o["gv0"])
    assert abs(g["gk"] - o["gk"]) <= GRAD_RTOL * abs(o["gk"]), (g["gk"], o["gk"])
    assert abs(g["gmu"] - o["gmu"]) <= GRAD_RTOL * abs(o["gmu"]), (g["gmu"], o["gmu"])


def test_adjoint_small_matches_fp64_oracle(cuda, olib):
    sc = differentiable_block(16, 16, 16)
    steps = 12
    tgt = target_positions(sc, steps)
    g = gpu_gradients(sc, steps, 5, tgt)
    o = oracle_gradients(olib, sc, steps, 5, tgt)
    check_against_oracle(g, o)
    assert field_rel(g["gp0"], o["gp0"]) < 1e-2, field_rel(g["gp0"], o["gp0"])


C5_STEPS, C5_EVERY = 200, 20


@pytest.fixture(scope="module")
def c5(cuda):
    """The differentiable rollout: 65,536 particles, 200 steps, checkpoint every 20."""
    sc = differentiable_block()
    tgt = target_positions(sc, C5_STEPS)
    return sc, tgt, gpu_gradients(sc, C5_STEPS, C5_EVERY, tgt)


def c5_loss(sc, tgt, vel=None, k=None, mu=None):
    import torch
    p = clone_params(sc.params)
    if k is not None:
        p.stiffness = k
    if mu is not None:
        p.viscosity = mu
        params_derive(p)
    f = make_fluid(sc, vel=vel, force=gravity4(sc))
    set_params(f, p)
    for _ in range(C5_STEPS):
        f.compute()
    torch.cuda.synchronize()
    x = f.getPositionBuffer().cpu().numpy().astype(np.float64)
    return float(np.mean((x[:, :3] - tgt[:, :3]) ** 2))


def gpu_states(sc, steps, vel=None):
    """(positions, velocities) before each of `steps` CUDA steps, float32 [steps, N, 4]."""
    import torch
    f = make_fluid(sc, vel=vel, force=gravity4(sc))
    sp, sv = [], []
    for _ in range(steps):
        sp.append(f.getPositionBuffer().cpu().numpy().copy())
        sv.append(f.getVelocityBuffer().cpu().numpy().copy())
        f.compute()
    torch.cuda.synchronize()
    return np.stack(sp), np.stack(sv), f.getPositionBuffer().cpu().numpy().astype(np.float64)


def test_adjoint_differentiable_block_same_trajectory(c5, olib):
    """The FP32 CUDA gradients with respect to v0, the gas constant and the viscosity within
    1e-3 of the FP64 adjoint evaluated along the same (CUDA) trajectory, whole 200 steps."""
    sc, tgt, g = c5
    sp, sv, final = gpu_states(sc, C5_STEPS)
    np.testing.assert_array_equal(final, g["pos"].astype(np.float64))  # the adjoint's forward is the plain step
    gpos = np.zeros((sc.n, 4))
    gpos[:, :3] = 2.0 * (final[:, :3] - tgt[:, :3]) / (3 * sc.n)
    gp0, gv0, gk, gmu = olib.adjoint_states_f64(sp, sv, gravity4(sc).astype(np.float64), sc.params, gpos)
    check_against_oracle(g, dict(gv0=gv0, gk=gk, gmu=gmu))
    assert field_rel(g["gp0"], gp0) < GRAD_RTOL, field_rel(g["gp0"], gp0)


def test_adjoint_differentiable_block_fp64_trajectory(c5, olib):
    """Against the FP64 oracle's own 200-step trajectory (which drifts from the FP32 one by
    about 1e-7): gradients with respect to v0, the gas constant and the viscosity within
    1e-3."""
    sc, tgt, g = c5
    o = oracle_gradients(olib, sc, C5_STEPS, C5_EVERY, tgt)
    check_against_oracle(g, o)


def floating_block(nx=64, ny=32, nz=32):
    """The differentiable block moved to the middle of its box: no particle meets a wall
    within 200 steps, so the loss is smooth in the parameters and initial velocities."""
    sc = differentiable_block(nx, ny, nz)
    ext = np.array([nx, ny, nz], np.float32) * 0.01
    sc.pos[:, :3] += 0.5 * ext
    return sc


@pytest.fixture(scope="module")
def floating(cuda):
    sc = floating_block()
    tgt = target_positions(sc, C5_STEPS)
    return sc, tgt, gpu_gradients(sc, C5_STEPS, C5_EVERY, tgt)


def test_adjoint_floating_block_fp64_trajectory(floating, olib):
    """The same against the FP64 oracle for the floating block (no wall contacts)."""
    sc, tgt, g = floating
    o = oracle_gradients(olib, sc, C5_STEPS, C5_EVERY, tgt)
    check_against_oracle(g, o)


def test_adjoint_matches_central_differences(floating):
    """Central differences (eps = 1e-3) of the CUDA forward rollout (200 steps, floating
    block): gas constant, viscosity and 16 random initial-velocity directions (each component
    moved by about 1e-3). The forward is FP32, so the differences carry rounding noise of a
    few 1e-3 relative; the bound is 5e-2 of the derivative's scale."""
    sc, tgt, g = floating
    eps = 1e-3
    k, mu = sc.params.stiffness, sc.params.viscosity
    fk = (c5_loss(sc, tgt, k=k + eps) - c5_loss(sc, tgt, k=k - eps)) / (2 * eps)
    fmu = (c5_loss(sc, tgt, mu=mu + eps) - c5_loss(sc, tgt, mu=mu - eps)) / (2 * eps)
    assert abs(g["gk"] - fk) <= 5e-2 * abs(fk), (g["gk"], fk)
    assert abs(g["gmu"] - fmu) <= 5e-2 * abs(fmu), (g["gmu"], fmu)
    rng = SplitMix64(17)
    gnorm = np.linalg.norm(g["gv0"][:, :3].astype(np.float64))
    for _ in range(16):
        d = np.zeros_like(sc.pos)
        d[:, :3] = rng.normal(3 * sc.n).reshape(sc.n, 3).astype(np.float32)
        fd = (c5_loss(sc, tgt, vel=(sc.vel + eps * d).astype(np.float32)) -
              c5_loss(sc, tgt, vel=(sc.vel - eps * d).astype(np.float32))) / (2 * eps)
        ad = float(np.sum(g["gv0"].astype(np.float64) * d))
        # a random direction's derivative is about |g|; judge the error on that scale
        assert abs(ad - fd) <= 5e-2 * max(abs(fd), gnorm), (ad, fd, gnorm)


def test_backward_is_deterministic_and_restores_state(cuda):
    import torch
    sc = differentiable_block(16, 16, 8)
    steps = 9
    tgt = target_positions(sc, steps)
    g = gpu_gradients(sc, steps, 4, tgt)
    f, adj = g["fluid"], g["adj"]
    np.testing.assert_array_equal(f.getPositionBuffer().cpu().numpy(), g["pos"])
    gpos = torch.from_numpy(np.ascontiguousarray(2.0 * (g["pos"] - tgt) / (3 * sc.n)).astype(np.float32)).cuda()
    gpos[:, 3] = 0
    a = adj.backward(gpos)
    b = adj.backward(gpos)
    torch.cuda.synchronize()
    for x, y in zip(a, b):
        assert torch.equal(x, y)
    np.testing.assert_array_equal(f.getPositionBuffer().cpu().numpy(), g["pos"])


def test_checkpoint_interval_does_not_change_gradients(cuda):
    import torch
    sc = differentiable_block(16, 16, 8)
    steps = 10
    tgt = target_positions(sc, steps)
    a = gpu_gradients(sc, steps, 3, tgt)
    b = gpu_gradients(sc, steps, 10, tgt)
    np.testing.assert_array_equal(a["gv0"], b["gv0"])
    np.testing.assert_array_equal(a["gp0"], b["gp0"])
    assert a["gk"] == b["gk"] and a["gmu"] == b["gmu"]


def test_autograd_rollout(cuda):
    """torch.autograd through libcl_gb300.autograd.rollout gives the adjoint's gradients."""
    import torch
    from libcl_gb300.autograd import rollout
    sc = differentiable_block(16, 16, 8)
    steps = 8
    tgt = torch.from_numpy(target_positions(sc, steps)).cuda()
    f = make_fluid(sc, force=gravity4(sc))
    adj = Adjoint3D(f, steps, 4)
    v0 = torch.from_numpy(sc.vel).cuda().requires_grad_(True)
    k = torch.tensor(sc.params.stiffness, dtype=torch.float64, requires_grad=True)
    mu = torch.tensor(sc.params.viscosity, dtype=torch.float64, requires_grad=True)
    pos0 = torch.from_numpy(sc.pos).cuda()
    x, _ = rollout(adj, pos0, v0, k, mu)

    def loss_of(xx):
        return torch.mean((xx[:, :3].double() - tgt[:, :3]) ** 2)

    gv, gk, gmu = torch.autograd.grad(loss_of(x), (v0, k, mu))
    # the same backward called directly with autograd's dL/dx
    xd = x.detach().clone().requires_grad_(True)
    (gx,) = torch.autograd.grad(loss_of(xd), (xd,))
    gp0, gv0, gpar = adj.backward(gx)
    torch.cuda.synchronize()
    assert torch.equal(gv, gv0)
    assert float(gk) == float(gpar[0]) and float(gmu) == float(gpar[1])
    # and the rollout's forward is the plain step
    ref = gpu_gradients(sc, steps, 4, tgt.cpu().numpy())
    np.testing.assert_array_equal(x.detach().cpu().numpy(), ref["pos"])
    np.testing.assert_allclose(gv.cpu().numpy(), ref["gv0"], rtol=1e-5, atol=1e-6 * np.abs(ref["gv0"]).max())


def test_adjoint_errors(cuda):
    import torch
    sc = differentiable_block(8, 8, 8)
    f = make_fluid(sc, force=gravity4(sc))
    adj = Adjoint3D(f, 4, 2)
    g = torch.zeros(sc.n, 4, device="cuda")
    with pytest.raises(GbsphError) as e:
        adj.backward(g)
    assert e.value.status == ERR_STATE
    adj.forward()
    f.getParameters().stiffness = 2.0
    with pytest.raises(GbsphError) as e:
        adj.backward(g)
    assert e.value.status == ERR_STATE
    f.getParameters().keyMode = KEY_REFERENCE_HASH
    with pytest.raises(GbsphError) as e:
        adj.forward()
    assert e.value.status == ERR_ARGUMENT
