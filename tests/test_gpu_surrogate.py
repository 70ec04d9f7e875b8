"""The learned-surrogate kernels on a GB300: training gradients against the NumPy
restatement, tensor-core inference against the FP32 path, and the surrogate
integrator against the plain integrator."""

from __future__ import annotations

import numpy as np
import pytest

from oracle import mlp_oracle as M
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    from galax_gb300.build import build

    build()
    import galax_gb300 as gx
    from galax_gb300 import surrogate as S

    return gx, S


def _params(S, seed=1, scale=1.0):
    p = S.init_params(seed)
    d = S.unpack(p)
    rng = np.random.default_rng(seed + 100)
    for k in ("b1", "b2", "b3", "b4"):
        d[k][:] = rng.normal(0, 0.1, d[k].shape)
    d["b5"][:] = 0.3
    return p * np.float32(scale) if scale != 1.0 else p


def _as_oracle(S, p):
    return {k: v.astype(np.float64) for k, v in S.unpack(p).items()}


def test_training_gradient_matches_numpy(env):
    gx, S = env
    p = _params(S)
    rng = np.random.default_rng(3)
    u = rng.normal(size=(96, 3)).astype(np.float32)
    pt = rng.normal(size=96).astype(np.float32)
    gt = rng.normal(size=(96, 3)).astype(np.float32)
    loss, grad = S.loss_grads(p, u, pt, gt, 0.7, 1.3, quantize=False)
    L_ref, g_ref = M.loss_and_grads(_as_oracle(S, p), u.astype(np.float64), pt.astype(np.float64),
                                    gt.astype(np.float64), 0.7, 1.3)
    assert abs(loss - L_ref) <= 1e-4 * abs(L_ref)
    gd = S.unpack(grad)
    for k in M.NAMES:
        ref = g_ref[k].reshape(-1)
        got = gd[k].reshape(-1).astype(np.float64)
        assert np.linalg.norm(got - ref) <= 2e-4 * np.linalg.norm(ref) + 1e-7, k


def test_weighted_training_gradient_matches_numpy(env):
    """Per-point loss weights (used to weight the far field) enter the exact gradient."""
    gx, S = env
    p = _params(S, seed=2)
    rng = np.random.default_rng(13)
    B = 2048  # above the split-K threshold of the weight-gradient products
    u = rng.normal(size=(B, 3)).astype(np.float32)
    pt = rng.normal(size=B).astype(np.float32)
    gt = rng.normal(size=(B, 3)).astype(np.float32)
    w = rng.uniform(0.1, 3.0, B).astype(np.float32)
    loss, grad = S.loss_grads(p, u, pt, gt, 0.4, 0.9, quantize=False, weights=w)
    L_ref, g_ref = M.loss_and_grads(_as_oracle(S, p), u.astype(np.float64), pt.astype(np.float64),
                                    gt.astype(np.float64), 0.4, 0.9, w.astype(np.float64))
    assert abs(loss - L_ref) <= 1e-4 * abs(L_ref)
    gd = S.unpack(grad)
    for k in M.NAMES:
        ref = g_ref[k].reshape(-1)
        got = gd[k].reshape(-1).astype(np.float64)
        assert np.linalg.norm(got - ref) <= 3e-4 * np.linalg.norm(ref) + 1e-7, k


@pytest.mark.parametrize("B", [1000, 4096])
def test_quantised_training_gradient_is_close_to_fp32(env, B):
    """The quantised pass (bf16 weights and activations, the products fed from
    bf16 images, the fused store phases, the two-term weight gradients) gives
    the FP32 gradient up to the bf16 rounding of its operands: a wrong image,
    orientation or term would be off by O(1). B = 1000 ends in a partial
    128-row block and a partial 64-row column-sum chunk; 4096 has several row
    blocks and the split-K weight gradients."""
    gx, S = env
    p = _params(S, seed=5)
    rng = np.random.default_rng(17)
    u = rng.normal(size=(B, 3)).astype(np.float32)
    pt = rng.normal(size=B).astype(np.float32)
    gt = rng.normal(size=(B, 3)).astype(np.float32)
    loss_q, grad_q = S.loss_grads(p, u, pt, gt, 0.7, 1.3, quantize=True)
    L_ref, g_ref = M.loss_and_grads(_as_oracle(S, p), u.astype(np.float64), pt.astype(np.float64),
                                    gt.astype(np.float64), 0.7, 1.3)
    assert abs(loss_q - L_ref) <= 2e-2 * abs(L_ref)
    gd = S.unpack(grad_q)
    for k in M.NAMES:
        ref = g_ref[k].reshape(-1)
        got = gd[k].reshape(-1).astype(np.float64)
        assert np.linalg.norm(got - ref) <= 5e-2 * np.linalg.norm(ref) + 1e-6, k


def test_quantised_fp32_forward_matches_numpy_bf16(env):
    gx, S = env
    p = _params(S)
    rng = np.random.default_rng(4)
    u = rng.normal(size=(512, 3)).astype(np.float32)
    mlp = S.MLPSurrogate(p, 1.0, 1.0)
    phi, g = mlp.forward_f32(u, quantize=True)
    out_ref, g_ref = M.forward_bf16(_as_oracle(S, p), u.astype(np.float64))
    phi, g = phi.cpu().numpy(), g.cpu().numpy()
    # bfloat16 rounding ties can fall differently with a different summation order
    assert np.median(np.abs(phi - out_ref)) < 1e-3 * np.abs(out_ref).mean()
    rel = np.linalg.norm(g - g_ref, axis=1) / np.linalg.norm(g_ref, axis=1)
    assert np.median(rel) < 5e-3 and rel.max() < 5e-2


@pytest.mark.parametrize("n", [300, 20000])
def test_tensor_core_inference_matches_fp32(env, n):
    import torch

    gx, S = env
    p = _params(S)
    length, pscale = 50.0, 3e-3
    mlp = S.MLPSurrogate(p, length, pscale)
    rng = np.random.default_rng(5)
    x = rng.normal(size=(n, 3)) * 30.0
    g, phi = mlp.evaluate(x, potential=True)
    phi_r, g_r = mlp.forward_f32(x / length, quantize=True)
    g_r = g_r.double().cpu().numpy() * (pscale / length)
    phi_r = phi_r.double().cpu().numpy() * pscale
    rel = np.linalg.norm(g - g_r, axis=1) / np.linalg.norm(g_r, axis=1)
    assert np.median(rel) < 5e-3 and np.percentile(rel, 99) < 3e-2
    assert np.median(np.abs(phi - phi_r)) < 2e-3 * np.abs(phi_r).mean()
    torch.cuda.synchronize()


@pytest.mark.parametrize("n", [300, 40000])
def test_tensor_core_inference_matches_numpy_bf16(env, n):
    """The tensor-core kernel against the NumPy restatement of the quantised
    network (oracle/mlp_oracle.py: bf16 weights and activations entering the
    256x256 products, FP32 accumulation), directly. Beyond bf16 rounding the
    kernel's sigmoid comes from one tanh.approx (~2^-11 relative) and its
    silu' is stored as bf16, so agreement is to a few bf16 units."""
    gx, S = env
    p = _params(S)
    length, pscale = 50.0, 3e-3
    mlp = S.MLPSurrogate(p, length, pscale)
    rng = np.random.default_rng(15)
    x = rng.normal(size=(n, 3)) * 30.0
    g, phi = mlp.evaluate(x, potential=True)
    out_r, g_r = M.forward_bf16(_as_oracle(S, p), x / length)
    g_r = g_r * (pscale / length)
    phi_r = out_r * pscale
    rel = np.linalg.norm(g - g_r, axis=1) / np.linalg.norm(g_r, axis=1)
    assert np.median(rel) < 5e-3 and np.percentile(rel, 99) < 3e-2
    assert np.median(np.abs(phi - phi_r)) < 2e-3 * np.abs(phi_r).mean()


def test_zero_network_surrogate_equals_plain_integrator(env):
    """With an MLP whose output is identically zero the surrogate integrator must
    reproduce the plain constant-step Dopri5 kernel on the analytic part, to
    rounding: the plain integrator compiles without implicit multiply-add
    contraction, the surrogate's stage kernels with it."""
    gx, S = env
    from galax_gb300 import workloads as W
    from galax_gb300.dynamics import integrate

    p = _params(S)
    d = S.unpack(p)
    d["w5"][:] = 0.0
    d["b5"][:] = 0.0
    mlp = S.MLPSurrogate(p, 50.0, 1e-3)
    mw = gx.MilkyWayPotential()
    y0 = W.disk_like_ics(lambda x: O.gradient(O.milky_way(), x), 1000, seed=8)
    for use_graph in (True, False):
        yT = S.integrate(mw, mlp, y0, 0.0, 100.0, 1.0, use_graph=use_graph).cpu().numpy()
        cfg = gx.Integrator(solver=gx.Dopri5(), stepsize_controller=gx.ConstantStepSize(), dt0=1.0).config()
        out, st, steps = integrate(mw, y0, 0.0, 100.0, np.array([100.0]), cfg)
        ref = out[:, 0, :].t().cpu().numpy()
        np.testing.assert_allclose(yT, ref, rtol=1e-12, atol=1e-15)


def test_surrogate_integrator_with_table_potential(env):
    """Analytic part as a general component table: the MLP term shifts the orbits."""
    gx, S = env
    from galax_gb300 import workloads as W

    p = _params(S, scale=0.5)
    mlp = S.MLPSurrogate(p, 50.0, 1e-4)
    kinds = gx.potential.from_component_array(O.milky_way()[[1, 0, 2, 3]])
    y0 = W.disk_like_ics(lambda x: O.gradient(O.milky_way(), x), 777, seed=9)
    a = S.integrate(kinds, None, y0, 0.0, 50.0, 1.0).cpu().numpy()
    b = S.integrate(kinds, mlp, y0, 0.0, 50.0, 1.0).cpu().numpy()
    ref, *_ = O.integrate(O.milky_way(), y0, 0.0, 50.0, np.array([50.0]), O.solver_cfg(5, False, dt0=1.0))
    np.testing.assert_allclose(a, np.stack(ref).reshape(-1, 6), rtol=1e-11, atol=1e-13)
    assert np.abs(b - a).max() > 1e-6


def test_training_reduces_the_loss(env):
    gx, S = env
    rng = np.random.default_rng(6)
    plum = O.comps([(O.PLUMMER, 5e9, 2.0, 0, (3.0, -1.0, 0.5))])
    r = np.exp(rng.uniform(np.log(0.5), np.log(40), 32768))
    v = rng.normal(size=(32768, 3))
    x = v / np.linalg.norm(v, axis=1, keepdims=True) * r[:, None]
    mlp, rep = S.train(x, O.potential(plum, x), O.gradient(plum, x), length_scale=20.0, epochs=40, batch=2048,
                       lr=2e-3)
    assert rep.loss[-1] < 0.25 * rep.loss[0]
    g = mlp.evaluate(x[:4096])
    g_ref = O.gradient(plum, x[:4096])
    rel = np.linalg.norm(g - g_ref, axis=1) / np.linalg.norm(g_ref, axis=1)
    assert np.median(rel) < 0.2


def _subhalos(n=64, seed=11):
    rng = np.random.default_rng(seed)
    m = np.exp(rng.uniform(np.log(1e6), np.log(1e8), n))
    b = rng.uniform(0.1, 1.0, n)
    v = rng.normal(size=(n, 3))
    c = v / np.linalg.norm(v, axis=1, keepdims=True) * rng.uniform(5.0, 30.0, n)[:, None]
    return O.comps([(O.PLUMMER, m[i], b[i], 0.0, tuple(c[i])) for i in range(n)])


def test_short_range_split_matches_direct_taper_sum(env):
    """The cell-list short-range sum equals the direct sum of the tapered spheres
    everywhere (next to centres, across cell faces, outside the grid) to the
    FP32 accuracy of its terms, measured against the untapered near-field scale:
    the centres and the point are held in FP32 relative to a cell corner
    (~1e-7 kpc absolute), which next to the most compact spheres (b = 0.1 kpc)
    is up to ~6e-6 of the gradient scale (an FP32 emulation of the kernel on
    these points gives 5.7e-6), and ~5e-7 for the potential."""
    gx, S = env
    subs = _subhalos()
    near = S.ShortRange(gx.potential.from_component_array(subs), 3.0)
    rng = np.random.default_rng(12)
    x = np.concatenate([
        rng.normal(size=(4000, 3)) * 20.0,                                              # spread out
        subs["origin"][rng.integers(0, len(subs), 4000)] + rng.normal(size=(4000, 3)),  # next to centres
        rng.normal(size=(50, 3)) * 200.0,                                               # mostly outside the grid
    ])
    phi, g = near.evaluate(x)
    phi_r, g_r, mphi, mg = O.plummer_short_range(subs, x, 3.0, magnitudes=True)
    phi, g = phi.cpu().numpy(), g.cpu().numpy()
    assert np.count_nonzero(phi_r) > 4000
    assert np.all(np.abs(phi - phi_r) <= 2e-6 * mphi + 1e-15 * mphi.max())
    assert np.all(np.linalg.norm(g - g_r, axis=1) <= 2e-5 * mg + 1e-15 * mg.max())
    far = np.linalg.norm(x, axis=1) > 150.0
    assert np.all(phi[far] == 0) and np.all(g[far] == 0)


def test_surrogate_integrator_adds_the_exact_short_range_field(env):
    """Zero MLP plus the split: the orbit is Dopri5 under Milky Way + short-range
    sum (checked against a NumPy constant-step Dopri5 on the oracle's FP64
    fields; the short-range terms are FP32, so agreement is to ~1e-8)."""
    gx, S = env
    from galax_gb300 import workloads as W

    subs = _subhalos(seed=14)
    near = S.ShortRange(gx.potential.from_component_array(subs), 4.0)
    p = _params(S)
    d = S.unpack(p)
    d["w5"][:] = 0.0
    d["b5"][:] = 0.0
    mlp = S.MLPSurrogate(p, 50.0, 1e-3)
    mw = gx.MilkyWayPotential()
    y0 = W.disk_like_ics(lambda x: O.gradient(O.milky_way(), x), 64, seed=15)
    got = S.integrate(mw, mlp, y0, 0.0, 60.0, 1.0, near=near).cpu().numpy()
    c, a, b, _ = O.tableau(5)

    def f(y):
        g = O.gradient(O.milky_way(), y[:, :3]) + O.plummer_short_range(subs, y[:, :3], 4.0)[1]
        return np.concatenate([y[:, 3:], -g], axis=1)

    y = y0.copy()
    for _ in range(60):
        F = [f(y)]
        for i in range(1, len(c)):
            F.append(f(y + sum(a[i][j] * F[j] for j in range(i)) * 1.0))
        y = y + sum(b[i] * F[i] for i in range(len(c))) * 1.0
    np.testing.assert_allclose(got, y, rtol=1e-7, atol=1e-9)
    plain = S.integrate(mw, mlp, y0, 0.0, 60.0, 1.0).cpu().numpy()
    assert np.abs(plain - got).max() > 1e-8  # the short-range field does act


def test_trained_surrogate_beats_the_analytic_part_alone(env):
    """What the learned part gains: orbits in the Milky Way plus 512 Plummer
    subhalos (the surrogate workload's composite) integrated for 1 Gyr with
    the analytic Milky Way alone, and with the Milky Way plus the near field
    plus a briefly trained MLP for the rest. Judged against the plain FP64
    direct sum over all 516 components, the trained network must cut the
    median relative position error at least tenfold."""
    import torch

    gx, S = env
    from galax_gb300 import workloads as W
    from galax_gb300.dynamics import integrate
    from galax_gb300.potential import from_component_array

    mw = gx.MilkyWayPotential()
    m, b, c = W.subhalo_table(3, 512)
    sub_arr = np.zeros(512, mw.component_array().dtype)
    sub_arr["kind"] = 4
    sub_arr["m"], sub_arr["l1"], sub_arr["origin"] = m, b, c
    sub = from_component_array(sub_arr)
    full = from_component_array(np.concatenate([mw.component_array(), sub_arr]))
    xt = torch.as_tensor(W.training_points(262_144, seed=30), device="cuda")
    near = S.ShortRange(sub, 12.0)
    ps, gs = near.evaluate(xt)
    mlp, rep = S.train(xt, sub.potential(xt) - ps, sub.gradient(xt) - gs, length_scale=50.0, epochs=60,
                       batch=8192, lr=2e-3)
    n, t1 = 2048, 1000.0
    y0 = torch.as_tensor(W.disk_like_ics(lambda x: O.gradient(O.milky_way(), x), n, seed=31), device="cuda")
    cfg = gx.Integrator(solver=gx.Dopri5(), stepsize_controller=gx.ConstantStepSize(), dt0=1.0).config()
    out, st, _ = integrate(full, y0.t().contiguous(), 0.0, t1, torch.tensor([t1]), cfg, soa=True)
    assert int((st != 0).sum()) == 0
    ref = out[:, 0, :].t()
    err = lambda y: (torch.linalg.vector_norm(y[:, :3] - ref[:, :3], dim=1)  # noqa: E731
                     / torch.linalg.vector_norm(ref[:, :3], dim=1))
    e_mw = float(err(S.integrate(mw, None, y0, 0.0, t1, 1.0)).median())
    e_sur = float(err(S.integrate(mw, mlp, y0, 0.0, t1, 1.0, near=near)).median())
    assert e_mw > 1e-2  # the subhalos matter
    assert e_sur < e_mw / 10, (e_sur, e_mw)


def test_training_is_deterministic(env):
    """Two trainings from the same seed give the same network bit for bit: the
    batches come from a keyed permutation, and the split-K weight gradients add
    their partial tiles in a fixed order."""
    gx, S = env
    rng = np.random.default_rng(16)
    plum = O.comps([(O.PLUMMER, 5e9, 2.0, 0, (3.0, -1.0, 0.5))])
    r = np.exp(rng.uniform(np.log(0.5), np.log(40), 16384))
    v = rng.normal(size=(16384, 3))
    x = v / np.linalg.norm(v, axis=1, keepdims=True) * r[:, None]
    phi, g = O.potential(plum, x), O.gradient(plum, x)
    a, ra = S.train(x, phi, g, length_scale=20.0, epochs=3, batch=8192, lr=2e-3)
    b, rb = S.train(x, phi, g, length_scale=20.0, epochs=3, batch=8192, lr=2e-3)
    np.testing.assert_array_equal(a.params, b.params)
