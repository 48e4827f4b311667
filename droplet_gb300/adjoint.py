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


def deformation_from_diag(d: dict, phi1: float, phi2: float):
    """D and the eigen data of the covariance of w from the device moments
    of dl_reduce (w_sum, w_x, w_xx = xx, yy, zz, xy, xz, yz)."""
    W = d["w_sum"]
    m = np.array(d["w_x"]) / W
    xx = np.array(d["w_xx"]) / W
    Cm = np.array([[xx[0], xx[3], xx[4]], [xx[3], xx[1], xx[5]], [xx[4], xx[5], xx[2]]]) - np.outer(m, m)
    lam, vec = np.linalg.eigh(Cm)
    la, lb = lam[-1], lam[0]
    A, B = math.sqrt(la), math.sqrt(lb)
    return (A - B) / (A + B), dict(W=W, m=m, la=la, lb=lb, va=vec[:, -1], vb=vec[:, 0], A=A, B=B)


class CheckpointedRun:
    """Forward and reverse passes of one FP32 run. When the per-step adjoint
    states of the whole run fit in `memory_fraction` of the free device memory
    (20 FP32 values per site and step, 35 with LES or a viscosity ratio; 35 GB
    for 500 steps of 96^3 with 20), the
    forward keeps all of them and the reverse pass recomputes nothing;
    otherwise it keeps a full state every S = ceil(sqrt(n)) steps and
    recomputes each segment once. The loss and its gradient stay on the
    device: D comes from the moments of dl_reduce, dD/dphi is formed from the
    coordinates and the eigen data."""

    def __init__(self, params: Params, shape, u0, p0, nsteps: int, segment: int | None = None,
                 memory_fraction: float = 0.6, force_mode: int = 0):
        import torch

        self.torch = torch
        self.params = params
        self.shape = tuple(shape)
        self.u0 = [np.ascontiguousarray(u, dtype=np.float64) for u in u0]
        self.p0 = np.ascontiguousarray(p0, dtype=np.float64)
        self.nsteps = int(nsteps)
        self.force_mode = int(force_mode)  # DL_FORCE_NONE or DL_FORCE_SPECTRAL (band forcing from u)
        self.timing = AdjointTiming()
        self.sim = None
        self._seg = None
        self.store_all = False
        if segment is None:
            nx, ny, nz = self.shape
            need = self.nsteps * (35 if (params.les or params.nu2 != params.nu1) else 20) * nx * ny * nz * 4
            free, _ = torch.cuda.mem_get_info()
            self.store_all = need <= memory_fraction * free
            segment = self.nsteps if self.store_all else max(1, math.ceil(math.sqrt(self.nsteps)))
        self.S = int(segment)

    def _buffer(self, kind: str):
        n = C.c_int64()
        fn = self.sim._lib.dl_state_floats if kind == "full" else self.sim._lib.dl_adjoint_state_floats
        rc = fn(self.sim._h, C.byref(n))
        if rc:
            raise RuntimeError(f"state size: {rc}")
        return self.torch.empty(int(n.value), dtype=self.torch.float32, device="cuda")

    def forward(self, phi0: np.ndarray) -> float:
        torch = self.torch
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        if self.sim is None:
            self.sim = Droplet(self.params, self.shape, FORM_FP32)
            # the pull form: every step's state is saved, and a push step's state
            # would need a settle launch before each save
            self.sim.set_option("push", 0)
            nck = 1 if self.store_all else (self.nsteps + self.S - 1) // self.S
            self.ckpt = [self._buffer("full") for _ in range(nck)]
            if self.store_all:
                n = self._buffer("adjoint").numel()
                self._all = torch.empty((self.nsteps, n), dtype=torch.float32, device="cuda")
        self.sim.step_count = 0
        self.sim.set_fields(phi0, self.u0[0], self.u0[1], self.u0[2], self.p0)
        self.sim.init_equilibrium()
        if self.force_mode:
            self.sim.set_force(self.force_mode)
        for k in range(self.nsteps):
            if k % self.S == 0:
                self.sim._call("save_state", C.c_void_p(self.ckpt[k // self.S].data_ptr()))
            if self.store_all:
                self.sim._call("save_adjoint_state", C.c_void_p(self._all[k].data_ptr()))
            self.sim.step(1)
        D, self.eig = deformation_from_diag(self.sim.reduce(), self.params.phi1, self.params.phi2)
        self.D = D
        self.timing.forward_s = time.perf_counter() - t0
        return D

    def loss_gradient(self):
        """dD/dphi at the final step as a device tensor (N floats, x fastest)."""
        torch = self.torch
        e = self.eig
        nx, ny, nz = self.shape
        dev = "cuda"
        X = torch.arange(nx, device=dev, dtype=torch.float64).view(1, 1, nx) - e["m"][0]
        Y = torch.arange(ny, device=dev, dtype=torch.float64).view(1, ny, 1) - e["m"][1]
        Z = torch.arange(nz, device=dev, dtype=torch.float64).view(nz, 1, 1) - e["m"][2]
        pa = X * e["va"][0] + Y * e["va"][1] + Z * e["va"][2]
        pb = X * e["vb"][0] + Y * e["vb"][1] + Z * e["vb"][2]
        A, B = e["A"], e["B"]
        dla = (2 * B / (A + B) ** 2) / (2 * A)
        dlb = (-2 * A / (A + B) ** 2) / (2 * B)
        g = (dla * (pa * pa - e["la"]) + dlb * (pb * pb - e["lb"])) / e["W"] / (self.params.phi2 - self.params.phi1)
        return g.to(torch.float32).reshape(-1).contiguous()

    def backward(self, dD_dphi=None, download: bool = True):
        """Returns dict with dphi0 (array, or device tensor when download is
        False), dkappaf, dkappag, dtauf, dmobility, dU."""
        torch = self.torch
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        if dD_dphi is None:
            lphi = self.loss_gradient()
        else:
            lphi = torch.as_tensor(np.ascontiguousarray(dD_dphi, dtype=np.float32).reshape(-1), device="cuda")
        self.sim._call("adjoint_begin", C.c_void_p(lphi.data_ptr()))
        if self.store_all:
            for k in range(self.nsteps - 1, -1, -1):
                self.sim._call("adjoint_step", C.c_void_p(self._all[k].data_ptr()), C.c_int64(k + 1))
        elif self._seg is None:
            self._seg = [self._buffer("adjoint") for _ in range(self.S)]
        seg = self._seg
        for j in ([] if self.store_all else reversed(range(len(self.ckpt)))):
            s0 = j * self.S
            s1 = min(s0 + self.S, self.nsteps)
            self.sim._call("load_state", C.c_void_p(self.ckpt[j].data_ptr()))
            self.sim.step_count = s0
            for k in range(s0, s1):
                self.sim._call("save_adjoint_state", C.c_void_p(seg[k - s0].data_ptr()))
                if k < s1 - 1:
                    self.sim.step(1)
            for k in range(s1 - 1, s0 - 1, -1):
                self.sim._call("adjoint_step", C.c_void_p(seg[k - s0].data_ptr()), C.c_int64(k + 1))
        out = torch.empty(self.sim.n_sites, dtype=torch.float32, device="cuda")
        self.sim._call("adjoint_init", C.c_void_p(self.ckpt[0].data_ptr()), C.c_void_p(out.data_ptr()))
        grads = (C.c_double * 4)()
        self.sim._call("adjoint_grads", grads)
        nz3 = (self.shape[2], self.shape[1], self.shape[0])
        dphi0 = out.double().cpu().numpy().reshape(nz3) if download else out.view(nz3)
        torch.cuda.synchronize()
        self.timing.backward_s = time.perf_counter() - t0
        return {"dphi0": dphi0, "dkappaf": grads[0], "dkappag": grads[1], "dtauf": grads[2],
                "dmobility": grads[2] / self.params.ds, "dU": grads[3]}

    def close(self):
        if self.sim is not None:
            self.sim.close()
            self.sim = None
        self.ckpt = []
        self._seg = None
        self._all = None


def _function():
    import torch

    class DropletDeformation(torch.autograd.Function):
        """D(phi0, kappaf, kappag, tauf, U) through n FP32 steps."""

        @staticmethod
        def forward(ctx, phi0, kappaf, kappag, tauf, wall_u, spec):
            P = spec["params"].replace(kappaf=float(kappaf), kappag=float(kappag), tauf=float(tauf),
                                       wall_u=(float(wall_u), 0.0, 0.0))
            run = CheckpointedRun(P, spec["shape"], spec["u0"], spec["p0"], spec["nsteps"], spec.get("segment"),
                                  force_mode=spec.get("force_mode", 0))
            D = run.forward(phi0.detach().double().cpu().numpy())
            ctx.run = run
            ctx.device = phi0.device
            return torch.tensor(D, dtype=torch.float64, device=phi0.device)

        @staticmethod
        def backward(ctx, gD):
            g = ctx.run.backward(download=False)
            ctx.run.close()
            s = gD.to(torch.float64)
            dphi0 = g["dphi0"].to(device=ctx.device, dtype=torch.float64) * s
            mk = lambda v: (torch.tensor(v, dtype=torch.float64, device=ctx.device) * s)  # noqa: E731
            return dphi0, mk(g["dkappaf"]), mk(g["dkappag"]), mk(g["dtauf"]), mk(g["dU"]), None

    return DropletDeformation


def deformation_loss(phi0, kappaf, kappag, tauf, wall_u, spec):
    """torch entry point: returns D as a 0-dim tensor; gradients flow to phi0,
    kappaf, kappag, tauf and wall_u. spec: params (Params template), shape
    (nx, ny, nz), u0 (three arrays), p0, nsteps[, segment][, force_mode]."""
    return _function().apply(phi0, kappaf, kappag, tauf, wall_u, spec)
