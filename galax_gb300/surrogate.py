"""Learned potential surrogate: an MLP stands in for an expensive composite.

For a composite such as MilkyWayPotential plus hundreds of Plummer subhalos,
the analytic part stays exact in FP64 and a small MLP (3 -> 256 -> 256 -> 256
-> 256 -> 1, SiLU) learns the expensive remainder (the subhalo sum) from FP64
samples of its potential and gradient. The MLP is trained on the GPU by the
library's own kernels (``gal_mlp_train_step``: forward, input gradient, the
exact loss gradient including the second-order terms, Adam) and evaluated by a
fused tensor-core kernel (``gal_mlp_eval``: BF16 weights, FP32 accumulation,
accumulators in TMEM). ``integrate`` advances orbits with the analytic FP64
gradient plus the MLP gradient (``gal_integrate_surrogate``).
"""

from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .dynamics import Workspace, _as_cuda
from .potential import AbstractPotential

HIDDEN = 256


def _torch():
    import torch

    return torch


def num_params() -> int:
    return int(_lib.load().gal_mlp_num_params())


def init_params(seed: int = 0) -> np.ndarray:
    """He-normal weights, zero biases, packed in the library's parameter order."""
    rng = np.random.default_rng(seed)
    parts = [
        rng.normal(0.0, math.sqrt(2.0 / 3), (HIDDEN, 3)), np.zeros(HIDDEN),
        rng.normal(0.0, math.sqrt(2.0 / HIDDEN), (HIDDEN, HIDDEN)), np.zeros(HIDDEN),
        rng.normal(0.0, math.sqrt(2.0 / HIDDEN), (HIDDEN, HIDDEN)), np.zeros(HIDDEN),
        rng.normal(0.0, math.sqrt(2.0 / HIDDEN), (HIDDEN, HIDDEN)), np.zeros(HIDDEN),
        rng.normal(0.0, math.sqrt(1.0 / HIDDEN), HIDDEN), np.zeros(1),
    ]
    p = np.concatenate([a.ravel() for a in parts]).astype(np.float32)
    assert p.size == num_params()
    return p


def unpack(p: np.ndarray) -> dict:
    """Parameter vector -> named arrays (W rows are output units)."""
    p = np.asarray(p)
    H = HIDDEN
    o = 0
    out = {}
    for name, shape in (("W1", (H, 3)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (H, H)), ("b3", (H,)),
                        ("W4", (H, H)), ("b4", (H,)), ("w5", (H,)), ("b5", (1,))):
        size = int(np.prod(shape))
        out[name] = p[o:o + size].reshape(shape)
        o += size
    return out


@dataclass
class TrainReport:
    steps: int
    epochs: int
    loss: list = field(default_factory=list)
    seconds: float = 0.0


class MLPSurrogate:
    """The trained network plus its unit scales: Phi(x) = phi_scale * out(x / length_scale)."""

    def __init__(self, params: np.ndarray, length_scale: float, phi_scale: float):
        self.params = np.ascontiguousarray(params, np.float32)
        self.length_scale = float(length_scale)
        self.phi_scale = float(phi_scale)
        self._handle = None
        self._dev = None

    # ---- inference on the tensor cores
    def handle(self) -> int:
        torch = _torch()
        dev = torch.cuda.current_device()
        if self._handle is None or self._dev != dev:
            self.release()
            L = _lib.load()
            h = C.c_void_p()
            _lib.check(L.gal_mlp_create(self.params.ctypes.data, self.length_scale, self.phi_scale, C.byref(h)),
                       "gal_mlp_create")
            self._handle, self._dev = h.value, dev
        return self._handle

    def release(self):
        if getattr(self, "_handle", None):
            try:
                _lib.load().gal_mlp_destroy(self._handle)
            except Exception:  # noqa: BLE001
                pass
        self._handle = None

    def __del__(self):
        self.release()

    def evaluate(self, x, *, potential: bool = False):
        """grad Phi (and Phi) at positions x (n, 3) in physical units, on the GPU."""
        torch = _torch()
        is_np = not isinstance(x, torch.Tensor)
        xs = _as_cuda(x, torch.float64).reshape(-1, 3).t().contiguous()
        n = xs.shape[1]
        g = torch.empty((3, n), dtype=torch.float64, device="cuda")
        phi = torch.empty(n, dtype=torch.float64, device="cuda") if potential else None
        L = _lib.load()
        st = torch.cuda.current_stream().cuda_stream
        _lib.check(L.gal_mlp_eval(self.handle(), xs.data_ptr(), n, g.data_ptr(), 0, 1.0,
                                  phi.data_ptr() if phi is not None else None, st), "gal_mlp_eval")
        code = C.c_int32()
        grad = g.t()
        if is_np:
            torch.cuda.synchronize()
            _lib.check(L.gal_mlp_error(self.handle(), C.byref(code)), "gal_mlp_error")
            if code.value:
                raise _lib.GalaxGB300Error(f"MLP inference kernel gave up waiting (code {code.value})")
            grad = grad.cpu().numpy()
            phi = phi.cpu().numpy() if phi is not None else None
        return (grad, phi) if potential else grad

    # ---- FP32 reference path (training numerics)
    def forward_f32(self, u, *, quantize: bool = True):
        """out(u), grad_u out(u) in network units with the FP32 training kernels."""
        torch = _torch()
        U = _as_cuda(u, torch.float32).reshape(-1, 3).contiguous()
        B = U.shape[0]
        P = torch.as_tensor(self.params, device="cuda")
        phi = torch.empty(B, dtype=torch.float32, device="cuda")
        g = torch.empty((B, 3), dtype=torch.float32, device="cuda")
        L = _lib.load()
        nb = C.c_size_t()
        _lib.check(L.gal_mlp_workspace_size(B, C.byref(nb)), "gal_mlp_workspace_size")
        ws = torch.zeros(nb.value, dtype=torch.uint8, device="cuda")
        st = torch.cuda.current_stream().cuda_stream
        _lib.check(L.gal_mlp_forward_f32(P.data_ptr(), U.data_ptr(), B, phi.data_ptr(), g.data_ptr(), int(quantize),
                                         ws.data_ptr(), ws.numel(), st), "gal_mlp_forward_f32")
        _check_ws(L, ws, B, st)
        return phi, g


def loss_grads(params, u, phi_t, g_t, alpha: float, beta: float, *, quantize: bool = False, weights=None):
    """Loss and its parameter gradient on the GPU (FP32), for checking."""
    torch = _torch()
    P = _as_cuda(params, torch.float32).contiguous()
    U = _as_cuda(u, torch.float32).reshape(-1, 3).contiguous()
    pt = _as_cuda(phi_t, torch.float32).reshape(-1).contiguous()
    gt = _as_cuda(g_t, torch.float32).reshape(-1, 3).contiguous()
    wt = _as_cuda(weights, torch.float32).reshape(-1).contiguous() if weights is not None else None
    B = U.shape[0]
    grad = torch.empty_like(P)
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    L = _lib.load()
    nb = C.c_size_t()
    _lib.check(L.gal_mlp_workspace_size(B, C.byref(nb)), "gal_mlp_workspace_size")
    ws = torch.zeros(nb.value, dtype=torch.uint8, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    _lib.check(L.gal_mlp_loss_grads(P.data_ptr(), U.data_ptr(), pt.data_ptr(), gt.data_ptr(),
                                    wt.data_ptr() if wt is not None else None, B, alpha, beta, int(quantize),
                                    grad.data_ptr(), loss.data_ptr(), ws.data_ptr(), ws.numel(), st),
               "gal_mlp_loss_grads")
    _check_ws(L, ws, B, st)
    return float(loss), grad.cpu().numpy()


def _check_ws(L, ws, batch: int, stream) -> None:
    code = C.c_int32()
    _lib.check(L.gal_mlp_workspace_error(ws.data_ptr(), batch, C.byref(code), stream), "gal_mlp_workspace_error")
    if code.value:
        raise _lib.GalaxGB300Error(f"MLP training kernels: a tensor-core product gave up waiting (code {code.value})")


def train(x, phi, grad, *, length_scale: float, epochs: int = 30, batch: int = 8192, lr: float = 2e-3,
          lr_final: float = 2e-5, alpha: float = 0.1, seed: int = 0, quantize: bool = True,
          far_field_weight: bool = False, log_every: int = 0) -> tuple[MLPSurrogate, TrainReport]:
    """Fit the MLP to FP64 samples (x (n,3), Phi (n,), grad Phi (n,3), physical
    units) with the GPU training kernels. phi_scale is set so the potential
    targets have unit variance; the gradient term is weighted by the inverse
    variance of its targets. Cosine learning-rate decay from lr to lr_final.

    far_field_weight: weight every point by 1 / (|g|^2 + g_med^2) (g_med the
    median gradient norm, the weights normalised to mean 1), so the squared
    error becomes a relative one: without it the few points next to a compact
    component, whose gradients are ~1000x the typical one, dominate the loss."""
    import time

    torch = _torch()
    xs = _as_cuda(x, torch.float64).reshape(-1, 3)
    ph = _as_cuda(phi, torch.float64).reshape(-1)
    gr = _as_cuda(grad, torch.float64).reshape(-1, 3)
    n = xs.shape[0]
    batch = min(batch, n)
    phi_scale = float(ph.std()) or 1.0
    u = (xs / length_scale).to(torch.float32)
    pt = (ph / phi_scale).to(torch.float32)
    gt = (gr * (length_scale / phi_scale)).to(torch.float32)
    beta = 1.0 / float((gt ** 2).sum(1).mean())
    wts = None
    if far_field_weight:
        g2 = (gt.double() ** 2).sum(1)
        w = 1.0 / (g2 + g2.median())
        wts = (w / w.mean()).to(torch.float32)
        beta = 1.0 / float((wts.double() * g2).mean())
    P = torch.as_tensor(init_params(seed), device="cuda")
    M = torch.zeros_like(P)
    V = torch.zeros_like(P)
    L = _lib.load()
    nb = C.c_size_t()
    _lib.check(L.gal_mlp_train_workspace_size(batch, C.byref(nb)), "gal_mlp_train_workspace_size")
    ws = torch.zeros(nb.value, dtype=torch.uint8, device="cuda")  # zeroed: it holds the error flag
    st = torch.cuda.current_stream().cuda_stream
    u, pt, gt = u.contiguous(), pt.contiguous(), gt.contiguous()
    wts = wts.contiguous() if wts is not None else None
    hist = torch.zeros(max(epochs, 1), dtype=torch.float32, device="cuda")
    rep = TrainReport(steps=(n // batch) * epochs, epochs=epochs)
    t0 = time.perf_counter()
    # whole epochs on the device: batches gathered through a keyed permutation,
    # one CUDA graph per step (gal_mlp_train)
    _lib.check(L.gal_mlp_train(P.data_ptr(), M.data_ptr(), V.data_ptr(), u.data_ptr(), pt.data_ptr(), gt.data_ptr(),
                               wts.data_ptr() if wts is not None else None, n, batch, epochs, alpha, beta, lr,
                               lr_final, 0.9, 0.999, 1e-8, seed, int(quantize), hist.data_ptr(), ws.data_ptr(),
                               ws.numel(), st), "gal_mlp_train")
    code = C.c_int32()
    _lib.check(L.gal_mlp_workspace_error(ws.data_ptr(), batch, C.byref(code), st), "gal_mlp_workspace_error")
    if code.value:
        raise _lib.GalaxGB300Error(f"MLP training: a tensor-core product gave up waiting (code {code.value})")
    rep.loss = hist[:epochs].cpu().tolist()
    if log_every:
        for ep in range(log_every - 1, epochs, log_every):
            print(f"epoch {ep + 1}: loss {rep.loss[ep]:.4e}", flush=True)
    rep.seconds = time.perf_counter() - t0
    return MLPSurrogate(P.cpu().numpy(), length_scale, phi_scale), rep


class ShortRange:
    """Exact FP64 short-range part of a set of Plummer spheres (``gal_split_*``).

    Every sphere is split as Phi S(d / r_cut) + Phi (1 - S), S(q) = (1 - q^2)^3
    for q < 1 (0 beyond): ``evaluate`` returns the short-range sum, which the
    surrogate integrator adds exactly; an MLP trained on ``total - short`` only
    has to learn the remainder, which is smooth on the scale r_cut."""

    def __init__(self, plummers: AbstractPotential, r_cut: float):
        arr = plummers.component_array()
        if np.any(arr["kind"] != _lib.GAL_PLUMMER):
            raise NotImplementedError("the short-range split takes Plummer components only")
        self.r_cut = float(r_cut)
        self._arr = np.ascontiguousarray(arr)
        self._G = plummers.G
        self._handle = None
        self._dev = None

    def handle(self) -> int:
        torch = _torch()
        dev = torch.cuda.current_device()
        if self._handle is None or self._dev != dev:
            self.release()
            h = C.c_void_p()
            _lib.check(_lib.load().gal_split_create(self._arr.ctypes.data, len(self._arr), self._G, self.r_cut,
                                                    C.byref(h)), "gal_split_create")
            self._handle, self._dev = h.value, dev
        return self._handle

    def release(self):
        if getattr(self, "_handle", None):
            try:
                _lib.load().gal_split_destroy(self._handle)
            except Exception:  # noqa: BLE001
                pass
        self._handle = None

    def __del__(self):
        self.release()

    def evaluate(self, x):
        """(phi (n,), grad (n, 3)) of the short-range part at x (n, 3), on the GPU."""
        torch = _torch()
        xs = _as_cuda(x, torch.float64).reshape(-1, 3).t().contiguous()
        n = xs.shape[1]
        phi = torch.empty(n, dtype=torch.float64, device="cuda")
        g = torch.empty((3, n), dtype=torch.float64, device="cuda")
        _lib.check(_lib.load().gal_split_eval(self.handle(), xs.data_ptr(), n, phi.data_ptr(), g.data_ptr(),
                                              torch.cuda.current_stream().cuda_stream), "gal_split_eval")
        return phi, g.t()


_WS = Workspace()


def integrate(analytic: AbstractPotential, mlp: MLPSurrogate | None, y0, t0: float, t1: float, dt: float, *,
              near: ShortRange | None = None, use_graph: bool = True, soa: bool = False):
    """Dopri5 with constant step dt under -grad(Phi_analytic + Phi_short + Phi_mlp)
    (``near`` the exact short-range part, or None); returns the final states
    (n, 6) (or (6, n) with soa=True), on the GPU."""
    torch = _torch()
    y = _as_cuda(y0, torch.float64)
    y = (y if soa else y.reshape(-1, 6).t()).contiguous().clone()
    n = y.shape[1]
    L = _lib.load()
    nb = C.c_size_t()
    _lib.check(L.gal_surrogate_workspace_size(n, C.byref(nb)), "gal_surrogate_workspace_size")
    ws = _WS.get(nb.value)
    st = torch.cuda.current_stream().cuda_stream
    _lib.check(L.gal_integrate_surrogate(analytic.handle(), mlp.handle() if mlp is not None else None,
                                         near.handle() if near is not None else None, float(dt), float(t0),
                                         float(t1), y.data_ptr(), n, int(use_graph), ws.data_ptr(), ws.numel(), st),
               "gal_integrate_surrogate")
    return y if soa else y.t()
