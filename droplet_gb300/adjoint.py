"""Gradients of the droplet deformation through the hand-written adjoint of
the FP32 step, behind a torch.autograd.Function, with sqrt(N) checkpointing.

Loss: D = (sqrt(l_max) - sqrt(l_min)) / (sqrt(l_max) + sqrt(l_min)) of the
covariance of w = (phi - phi1)/(phi2 - phi1) = (1 + phi~)/2 at the final step
(the 3-D form of the inertia-tensor measure of
prototype_program/two-phase/drop8_mpi.f90:812-970).

Differentiable inputs: the initial phi, kappaf, kappag, tau_f (the mobility is
(tau_f - 1/2) ds) and the wall velocity U (top wall +U, bottom wall -U in x).

Checkpointing: the forward keeps the device state every S = ceil(sqrt(n))
steps; the backward reloads each segment's checkpoint, recomputes the segment
keeping every state, and runs dl_adjoint_step over it in reverse; finally
dl_adjoint_init carries the adjoint through f = feq(phi0), g = geq(phi0).
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import math
import time

import numpy as np

from . import _abi
from .params import Params
from .solver import Droplet, FORM_FP32


def deformation_and_grad(phi: np.ndarray, phi1: float, phi2: float):
    """D of the covariance of w and dD/dphi (both float64)."""
    nz, ny, nx = phi.shape
    z, y, x = np.meshgrid(np.arange(nz, dtype=np.float64), np.arange(ny, dtype=np.float64),
                          np.arange(nx, dtype=np.float64), indexing="ij")
    w = (phi - phi1) / (phi2 - phi1)
    W = w.sum()
    X = [x, y, z]
    m = np.array([(w * c).sum() / W for c in X])
    Cm = np.empty((3, 3))
    for a in range(3):
        for b in range(3):
            Cm[a, b] = (w * X[a] * X[b]).sum() / W - m[a] * m[b]
    lam, vec = np.linalg.eigh(Cm)
    la, lb = lam[-1], lam[0]
    A, B = math.sqrt(la), math.sqrt(lb)
    D = (A - B) / (A + B)
    dD_dla = (2 * B / (A + B) ** 2) / (2 * A)
    dD_dlb = (-2 * A / (A + B) ** 2) / (2 * B)
    d = [X[k] - m[k] for k in range(3)]
    proj_a = sum(vec[k, -1] * d[k] for k in range(3))
    proj_b = sum(vec[k, 0] * d[k] for k in range(3))
    dD_dw = (dD_dla * (proj_a ** 2 - la) + dD_dlb * (proj_b ** 2 - lb)) / W
    return D, dD_dw / (phi2 - phi1)


@dataclasses.dataclass
class AdjointTiming:
    forward_s: float = 0.0
    backward_s: float = 0.0

    @property
    def ratio(self) -> float:
        return self.backward_s / self.forward_s if self.forward_s > 0 else float("nan")


class CheckpointedRun:
    """Forward and reverse passes of one FP32 run with sqrt(n) checkpoints."""

    def __init__(self, params: Params, shape, u0, p0, nsteps: int, segment: int | None = None):
        import torch

        self.torch = torch
        self.params = params
        self.shape = tuple(shape)
        self.u0 = [np.ascontiguousarray(u, dtype=np.float64) for u in u0]
        self.p0 = np.ascontiguousarray(p0, dtype=np.float64)
        self.nsteps = int(nsteps)
        self.S = int(segment or max(1, math.ceil(math.sqrt(self.nsteps))))
        self.timing = AdjointTiming()
        self.sim = None

    def _state_buffer(self):
        n = C.c_int64()
        rc = self.sim._lib.dl_state_floats(self.sim._h, C.byref(n))
        if rc:
            raise RuntimeError(f"dl_state_floats: {rc}")
        return self.torch.empty(int(n.value), dtype=self.torch.float32, device="cuda")

    def _save(self, buf):
        self.sim._call("save_state", C.c_void_p(buf.data_ptr()))

    def _load(self, buf):
        self.sim._call("load_state", C.c_void_p(buf.data_ptr()))

    def forward(self, phi0: np.ndarray) -> float:
        torch = self.torch
        t0 = time.perf_counter()
        if self.sim is not None:
            self.sim.close()
        self.sim = Droplet(self.params, self.shape, FORM_FP32)
        self.sim.set_fields(phi0, self.u0[0], self.u0[1], self.u0[2], self.p0)
        self.sim.init_equilibrium()
        self.ckpt = []
        for k in range(self.nsteps):
            if k % self.S == 0:
                b = self._state_buffer()
                self._save(b)
                self.ckpt.append(b)
            self.sim.step(1)
        f = self.sim.get_fields()
        torch.cuda.synchronize()
        self.timing.forward_s = time.perf_counter() - t0
        self.phi_final = f["phi"]
        D, self.dD_dphi = deformation_and_grad(f["phi"], self.params.phi1, self.params.phi2)
        self.D = D
        return D

    def backward(self, dD_dphi: np.ndarray | None = None):
        """Returns dict with dphi0 (array), dkappaf, dkappag, dtauf, dU."""
        torch = self.torch
        t0 = time.perf_counter()
        g = self.dD_dphi if dD_dphi is None else dD_dphi
        lphi = torch.tensor(np.ascontiguousarray(g, dtype=np.float32).reshape(-1), device="cuda")
        self.sim._call("adjoint_begin", C.c_void_p(lphi.data_ptr()))
        nseg = len(self.ckpt)
        seg_states = [self._state_buffer() for _ in range(self.S)]
        for j in reversed(range(nseg)):
            s0 = j * self.S
            s1 = min(s0 + self.S, self.nsteps)
            self._load(self.ckpt[j])
            self.sim.step_count = s0
            seg_states[0].copy_(self.ckpt[j])
            for k in range(s0, s1 - 1):
                self.sim.step(1)
                self._save(seg_states[k + 1 - s0])
            for k in range(s1 - 1, s0 - 1, -1):
                self.sim._call("adjoint_step", C.c_void_p(seg_states[k - s0].data_ptr()), C.c_int64(k + 1))
        out = torch.empty(self.sim.n_sites, dtype=torch.float32, device="cuda")
        self.sim._call("adjoint_init", C.c_void_p(self.ckpt[0].data_ptr()), C.c_void_p(out.data_ptr()))
        grads = (C.c_double * 4)()
        self.sim._call("adjoint_grads", grads)
        dphi0 = out.double().cpu().numpy().reshape(self.shape[2], self.shape[1], self.shape[0])
        torch.cuda.synchronize()
        self.timing.backward_s = time.perf_counter() - t0
        return {"dphi0": dphi0, "dkappaf": grads[0], "dkappag": grads[1], "dtauf": grads[2],
                "dmobility": grads[2] / self.params.ds, "dU": grads[3]}

    def close(self):
        if self.sim is not None:
            self.sim.close()
            self.sim = None


def _function():
    import torch

    class DropletDeformation(torch.autograd.Function):
        """D(phi0, kappaf, kappag, tauf, U) through n FP32 steps."""

        @staticmethod
        def forward(ctx, phi0, kappaf, kappag, tauf, wall_u, spec):
            P = spec["params"].replace(kappaf=float(kappaf), kappag=float(kappag), tauf=float(tauf),
                                       wall_u=(float(wall_u), 0.0, 0.0))
            run = CheckpointedRun(P, spec["shape"], spec["u0"], spec["p0"], spec["nsteps"], spec.get("segment"))
            D = run.forward(phi0.detach().double().cpu().numpy())
            ctx.run = run
            ctx.device = phi0.device
            return torch.tensor(D, dtype=torch.float64, device=phi0.device)

        @staticmethod
        def backward(ctx, gD):
            g = ctx.run.backward()
            ctx.run.close()
            s = gD.to(torch.float64)
            dphi0 = torch.tensor(g["dphi0"], device=ctx.device) * s
            mk = lambda v: (torch.tensor(v, dtype=torch.float64, device=ctx.device) * s)  # noqa: E731
            return dphi0, mk(g["dkappaf"]), mk(g["dkappag"]), mk(g["dtauf"]), mk(g["dU"]), None

    return DropletDeformation


def deformation_loss(phi0, kappaf, kappag, tauf, wall_u, spec):
    """torch entry point: returns D as a 0-dim tensor; gradients flow to phi0,
    kappaf, kappag, tauf and wall_u. spec: params (Params template), shape
    (nx, ny, nz), u0 (three arrays), p0, nsteps[, segment]."""
    return _function().apply(phi0, kappaf, kappag, tauf, wall_u, spec)
