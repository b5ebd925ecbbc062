"""Learned force surrogate for expensive potentials (the spherical-harmonic
expansion): an MLP (x, y, z, ln r) -> Phi with 4 hidden SiLU layers of width
128, trained on the GPU by the library's own kernels (ss_mlp_loss_grad:
value + force loss differentiated through the network's input gradient;
ss_mlp_adam), evaluated in FP32 on CUDA cores (ss_mlp_eval) or with BF16
weights on the tensor cores inside the stream integrator
(ss_stream_mlp_bf16).  The exact potential stays the reference: it makes
the training set and measures the surrogate's error.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field
from typing import Optional

import numpy as np
import torch

from . import _abi, _core
from ._core import ptr, stream_handle

NPARAM = _abi.SS_MLP_NPARAM
W = _abi.SS_MLP_WIDTH
# packed offsets (W[out][in])
OFF = {"W1": 0, "b1": 512, "W2": 640, "b2": 640 + 16384, "W3": 640 + 16384 + 128,
       "b3": 640 + 2 * 16384 + 128, "W4": 640 + 2 * 16384 + 256, "b4": 640 + 3 * 16384 + 256,
       "w5": 640 + 3 * 16384 + 384, "b5": 640 + 3 * 16384 + 512}


def unpack(params: torch.Tensor) -> dict:
    """Views of the packed parameter vector as matrices / vectors."""
    p = params
    return {"W1": p[0:512].view(W, 4), "b1": p[512:640],
            "W2": p[OFF["W2"]:OFF["b2"]].view(W, W), "b2": p[OFF["b2"]:OFF["W3"]],
            "W3": p[OFF["W3"]:OFF["b3"]].view(W, W), "b3": p[OFF["b3"]:OFF["W4"]],
            "W4": p[OFF["W4"]:OFF["b4"]].view(W, W), "b4": p[OFF["b4"]:OFF["w5"]],
            "w5": p[OFF["w5"]:OFF["b5"]], "b5": p[OFF["b5"]:OFF["b5"] + 1]}


@dataclass
class MLPSurrogate:
    params: torch.Tensor                 # [NPARAM] float32 (device)
    in_scale: tuple = (1.0, 1.0, 1.0, 1.0)
    in_shift: tuple = (0.0, 0.0, 0.0, 0.0)
    out_scale: float = 1.0
    out_shift: float = 0.0
    history: list = field(default_factory=list)
    # exact spherical part Phi_0(r) added to the network (ss_mlp.base): a
    # [n, 2] float64 device table of (value, d/du) at u = base_u0 + k base_du,
    # u = ln r; None = the network alone
    base: Optional[torch.Tensor] = None
    base_u0: float = 0.0
    base_du: float = 1.0

    @staticmethod
    def init(seed=0, in_scale=(1.0, 1.0, 1.0, 1.0), in_shift=(0.0, 0.0, 0.0, 0.0), out_scale=1.0, out_shift=0.0,
             device=None) -> "MLPSurrogate":
        """Random initialisation: W ~ N(0, 1/fan_in), zero biases."""
        g = torch.Generator().manual_seed(seed)
        p = torch.zeros(NPARAM, dtype=torch.float32)
        v = unpack(p)
        v["W1"].copy_(torch.randn(W, 4, generator=g) / math.sqrt(4.0))
        for k in ("W2", "W3", "W4"):
            v[k].copy_(torch.randn(W, W, generator=g) / math.sqrt(W))
        v["w5"].copy_(torch.randn(W, generator=g) / math.sqrt(W))
        return MLPSurrogate(p.to(device or _core.device()), tuple(in_scale), tuple(in_shift), float(out_scale),
                            float(out_shift))

    def struct(self) -> _abi.ss_mlp:
        m = _abi.ss_mlp()
        m.params = self.params.data_ptr()
        for i in range(4):
            m.in_scale[i] = float(self.in_scale[i])
            m.in_shift[i] = float(self.in_shift[i])
        m.out_scale = float(self.out_scale)
        m.out_shift = float(self.out_shift)
        if self.base is not None:
            m.base = self.base.data_ptr()
            m.base_n = int(self.base.shape[0])
            m.base_u0 = float(self.base_u0)
            m.base_du = float(self.base_du)
        return m

    @staticmethod
    def monopole_of(pot):
        """(table [n, 2], u0, du) of the l = 0 term of a spherical-harmonic
        expansion potential: its exact spherical part."""
        coef = pot.coef.to(_core.device(), torch.float64)
        return (float(pot.scale) * coef[:, 0, :]).contiguous(), float(pot.log_r0), float(pot.dlog_r)

    def with_base(self, base, u0, du) -> "MLPSurrogate":
        """Add the exact spherical part (ss_mlp.base); returns self."""
        self.base = base.to(_core.device(), torch.float64).contiguous()
        self.base_u0, self.base_du = float(u0), float(du)
        return self

    # ---------------------------------------------------------- evaluation
    def potential_and_gradient(self, xyz):
        """FP32 CUDA-core evaluation: (Phi [n], grad Phi [n,3]) float64."""
        x = _core.f64(xyz).reshape(-1, 3).contiguous()
        n = x.shape[0]
        phi = torch.empty(n, dtype=torch.float64, device=x.device)
        grad = torch.empty(n, 3, dtype=torch.float64, device=x.device)
        m = self.struct()
        need = _abi.load().ss_mlp_eval_workspace_bytes(n)
        ws, nb = _core.aligned_ptr(_core.Workspace.get(need, x.device, "mlp"))
        _abi.call("ss_mlp_eval", C.byref(m), ptr(x), n, ptr(phi), ptr(grad), ws, nb, stream_handle())
        return phi, grad

    def gradient_bf16(self, xyz):
        """grad Phi through the tensor-core path of the stream integrator."""
        x = _core.f64(xyz).reshape(-1, 3).contiguous()
        n = x.shape[0]
        grad = torch.empty(n, 3, dtype=torch.float64, device=x.device)
        st = torch.empty(n, dtype=torch.int32, device=x.device)
        m = self.struct()
        _abi.call("ss_mlp_grad_bf16", C.byref(m), ptr(x), n, ptr(grad), ptr(st), stream_handle())
        if bool((st != 0).any()):
            raise RuntimeError("ss_mlp_grad_bf16: a tensor-core wait timed out")
        return grad

    def loss_grad(self, x, phi_t, g_t, w_val, w_force):
        """(loss [2] = (value part, force part), grad [NPARAM]) of one batch."""
        B = x.shape[0]
        loss = torch.empty(2, dtype=torch.float32, device=x.device)
        grad = torch.empty(NPARAM, dtype=torch.float32, device=x.device)
        m = self.struct()
        need = _abi.load().ss_mlp_train_workspace_bytes(B)
        ws, nb = _core.aligned_ptr(_core.Workspace.get(need, x.device, "mlp_train"))
        _abi.call("ss_mlp_loss_grad", C.byref(m), ptr(x), ptr(phi_t), ptr(g_t), ptr(w_val), ptr(w_force), B,
                  ptr(loss), ptr(grad), ws, nb, stream_handle())
        return loss, grad

    # ------------------------------------------------------------ training
    def fit(self, x, phi, grad, steps=4000, batch=8192, lr=2e-3, lr_min=2e-5, force_weight=1.0, seed=0,
            log_every=0, force_scale=None):
        """Adam on the value + force loss with cosine learning-rate decay.
        x [N,3], phi [N], grad [N,3] (exact targets, any float dtype).  The
        force loss is relative: each sample's force error is divided by
        force_scale [N] (default |grad|; a residual fit passes the total
        force's magnitude, so that it minimises the error of the sum)."""
        dev = self.params.device
        x = x.to(dev, torch.float32).contiguous()
        phi = phi.to(dev, torch.float32).contiguous()
        N = x.shape[0]
        batch = min(batch, N)
        if force_scale is None:
            gnorm2 = (grad.double() ** 2).sum(1).clamp_min(1e-300)
        else:
            gnorm2 = (force_scale.to(dev, torch.float64) ** 2).clamp_min(1e-300)
        grad = grad.to(dev, torch.float32).contiguous()
        w_val_all = torch.full((N,), 1.0 / (batch * self.out_scale ** 2), dtype=torch.float32, device=dev)
        w_force_all = (force_weight / (batch * gnorm2)).float().contiguous()
        m = torch.zeros_like(self.params)
        v = torch.zeros_like(self.params)
        # the batches: consecutive slices of a fresh permutation per pass over
        # the set (the last partial slice of a pass is dropped)
        gen = torch.Generator(device=dev).manual_seed(seed)
        per_pass = N // batch
        parts, have = [], 0
        while have < steps:
            parts.append(torch.randperm(N, generator=gen, device=dev)[:per_pass * batch])
            have += per_pass
        order = torch.cat(parts)[:steps * batch].to(torch.int32).contiguous()
        log = torch.empty(max(steps, 1), 2, dtype=torch.float32, device=dev)
        lib = _abi.load()
        need = lib.ss_mlp_fit_workspace_bytes(batch)
        ws, nb = _core.aligned_ptr(_core.Workspace.get(need, dev, "mlp_fit"))
        st = self.struct()
        _abi.call("ss_mlp_fit", C.byref(st), ptr(self.params), ptr(x), ptr(phi), ptr(grad), ptr(w_val_all),
                  ptr(w_force_all), N, ptr(order), batch, steps, C.c_float(lr), C.c_float(lr_min), C.c_float(0.9),
                  C.c_float(0.999), C.c_float(1e-8), ptr(m), ptr(v), ptr(log), ws, nb, stream_handle())
        if log_every and steps:
            logged = [it for it in range(1, steps + 1) if it % log_every == 0 or it == steps]
            lh = log[torch.as_tensor([it - 1 for it in logged], device=dev)].cpu().numpy()
            self.history.extend((it, float(a), float(b)) for it, (a, b) in zip(logged, lh))
        return self

    @staticmethod
    def normalisation(x, phi):
        """Input / output affine maps from a training set."""
        x = torch.as_tensor(x, dtype=torch.float64)
        phi = torch.as_tensor(phi, dtype=torch.float64)
        L = float(x.abs().mean()) * 1.5
        lr = 0.5 * torch.log((x ** 2).sum(1))
        return dict(in_scale=(1.0 / L, 1.0 / L, 1.0 / L, 1.0 / float(lr.std())),
                    in_shift=(0.0, 0.0, 0.0, float(lr.mean())),
                    out_scale=float(phi.std()), out_shift=float(phi.mean()))


def orbit_samples(pot, prog_w0, n_orbits=4096, n_per_orbit=1024, dt=1.0, every=2, seed=0, broad_fraction=0.25):
    """Training points along orbits in `pot` (FP64 orbit kernel): most
    orbits start near the progenitor's orbit (position scatter 2 kpc,
    velocity scatter 10 % + 0.02 kpc/Myr), the rest isotropically with
    ln r uniform over [ln 1, ln 100] kpc and speeds of 0.3-1.2 times the
    circular speed.  Returns positions [n_orbits * n_per_orbit, 3] (float64)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    n_near = int(round(n_orbits * (1.0 - broad_fraction)))
    n_broad = n_orbits - n_near
    w0 = np.asarray(prog_w0, dtype=np.float64)
    T = n_per_orbit * every * dt
    prog = pot.integrate_orbit(w0=w0, ts=np.linspace(0.0, -T, 257), t0=0.0, t1=-T, dt=dt).ys
    prog = prog.detach().cpu().numpy()
    pick = prog[rng.integers(0, len(prog), n_near)]
    near = pick.copy()
    near[:, :3] += rng.normal(0.0, 2.0, (n_near, 3))
    near[:, 3:] = near[:, 3:] * (1.0 + rng.normal(0.0, 0.1, (n_near, 1))) + rng.normal(0.0, 0.02, (n_near, 3))
    r = np.exp(rng.uniform(np.log(1.0), np.log(100.0), n_broad))
    u = rng.normal(size=(n_broad, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    pos = u * r[:, None]
    g = pot.gradient(pos, 0.0).detach().cpu().numpy()
    vc = np.sqrt(np.maximum((g * pos).sum(1), 1e-30))
    d = rng.normal(size=(n_broad, 3))
    d -= (d * u).sum(1, keepdims=True) * u
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    vel = d * (vc * rng.uniform(0.3, 1.2, n_broad))[:, None]
    ics = np.concatenate([near, np.concatenate([pos, vel], 1)], 0)
    w = _core.f64(ics).contiguous()
    ys = _core.orbit(pot._desc(), w, 0.0, float(dt), n_per_orbit * every, every, method="serial")
    return ys[:, 1:, :3].reshape(-1, 3).contiguous()


def residual_targets(pot, x):
    """Phi and grad Phi of an expansion potential at x minus its exact
    spherical part (the l = 0 term, evaluated by the same FP64 kernels as a
    one-term expansion), and that part's table: what a surrogate with an
    exact base is trained on."""
    from .potential import SphericalHarmonicExpansionPotential
    table, u0, du = MLPSurrogate.monopole_of(pot)
    mono = SphericalHarmonicExpansionPotential(pot.coef[:, :1, :], pot.log_r0, pot.dlog_r, scale=pot.scale,
                                               units=pot.units)
    phi = pot.potential(x, 0.0) - mono.potential(x, 0.0)
    grad = pot.gradient(x, 0.0) - mono.gradient(x, 0.0)
    return phi, grad, (table, u0, du)


def train_surrogate(pot, prog_w0, n_points=1 << 22, steps=6000, batch=8192, seed=0, residual=None,
                    **kw) -> MLPSurrogate:
    """Sample `n_points` along orbits of the exact potential, evaluate Phi and
    grad Phi there with the exact FP64 kernels, and fit the network.  For an
    expansion potential (residual=None or True) the network learns the
    residual Phi - Phi_0 and the l = 0 term Phi_0 is added exactly, so the
    network's error multiplies only the anisotropic part; the force loss is
    relative to the total force."""
    from .potential import SphericalHarmonicExpansionPotential
    n_per = 1024
    n_orb = max(1, n_points // n_per)
    x = orbit_samples(pot, prog_w0, n_orbits=n_orb, n_per_orbit=n_per, seed=seed)
    if residual is None:
        residual = isinstance(pot, SphericalHarmonicExpansionPotential)
    base, scale = None, None
    if residual:
        phi, grad, base = residual_targets(pot, x)
        scale = torch.linalg.norm(pot.gradient(x, 0.0), dim=1)
    else:
        phi, grad = pot.potential(x, 0.0), pot.gradient(x, 0.0)
    nm = MLPSurrogate.normalisation(x.cpu(), phi.cpu())
    s = MLPSurrogate.init(seed=seed, **nm)
    if base is not None:
        s.with_base(*base)
    s.fit(x, phi, grad, steps=steps, batch=batch, seed=seed, force_scale=scale, **kw)
    return s
