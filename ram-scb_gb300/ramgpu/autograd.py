"""PyTorch autograd wrapper of the adjoint C-ABI pair.

``window_misfit(gpu, f2, fgeos, ...)`` returns J per member for a window of
ram_run calls starting from the state ``f2`` with boundary ``fgeos``;
``J.sum().backward()`` (or any upstream gradient) then runs
``ramgpu_adj_backward`` and delivers dJ/dF2 and dJ/dFGEOS in ``f2.grad`` and
``fgeos.grad``.  Both tensors are float64 CUDA tensors in the library's
device layout:

  f2    : (members, NS, NPA, NE, NT, NR)   F2(S,I,J,K,L) with I fastest
  fgeos : (members, NS, NPA, NE, NT)       FGEOS(S,J,K,L) with J fastest

Slots of species a member does not carry are ignored on the way in and get
zero gradient.  The device copies go through ramgpu_upload_f2 /
ramgpu_set_boundary / ramgpu_adj_backward with device pointers (unified
addressing), so no host round trip is made.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from .abi import RamGpu, _P


def _ptr(t: torch.Tensor):
    return C.cast(C.c_void_p(t.data_ptr()), _P)


class _WindowMisfit(torch.autograd.Function):
    @staticmethod
    def forward(ctx, f2, fgeos, gpu: RamGpu, ncalls, dts, kp, k_ckpt, obs):
        g = gpu.grid
        want = (gpu.n_members, gpu.ns, g.npa, g.ne, g.nt, g.nr)
        if tuple(f2.shape) != want or tuple(fgeos.shape) != want[:-1]:
            raise ValueError(f"f2 must be {want} and fgeos {want[:-1]}")
        if f2.dtype != torch.float64 or fgeos.dtype != torch.float64 or not f2.is_cuda:
            raise ValueError("f2 and fgeos must be float64 CUDA tensors")
        f2c, fgc = f2.detach().contiguous(), fgeos.detach().contiguous()
        torch.cuda.synchronize(f2.device)
        for m in range(gpu.n_members):
            for s in gpu.member_species[m]:
                gpu._ck(gpu.lib.ramgpu_upload_f2(gpu.h, m, s, _ptr(f2c[m, s])), "upload_f2")
                gpu._ck(gpu.lib.ramgpu_set_boundary(gpu.h, m, s, _ptr(fgc[m, s])), "set_boundary")
        J = gpu.adj_forward(ncalls, dts, kp, k_ckpt, obs)
        ctx.gpu = gpu
        ctx.shapes = (f2.shape, fgeos.shape, f2.device)
        return torch.as_tensor(J, dtype=torch.float64, device=f2.device)

    @staticmethod
    def backward(ctx, gJ):
        gpu = ctx.gpu
        sf, sb, dev = ctx.shapes
        gf = torch.empty(sf, dtype=torch.float64, device=dev)
        gb = torch.empty(sb, dtype=torch.float64, device=dev)
        torch.cuda.synchronize(dev)
        gpu._ck(gpu.lib.ramgpu_adj_backward(gpu.h, _ptr(gf), _ptr(gb)), "adj_backward")
        w = gJ.to(torch.float64).reshape(-1, 1, 1, 1, 1, 1)
        return gf * w, gb * w.reshape(-1, 1, 1, 1, 1), None, None, None, None, None, None


def window_misfit(gpu: RamGpu, f2: torch.Tensor, fgeos: torch.Tensor, ncalls: int, dts: float, kp,
                  k_ckpt: int, obs) -> torch.Tensor:
    """J per member (a differentiable tensor of shape (members,))."""
    return _WindowMisfit.apply(f2, fgeos, gpu, int(ncalls), float(dts), np.asarray(kp, dtype=np.float64),
                               int(k_ckpt), list(obs))


def device_state(gpu: RamGpu, f2_list, fgeos_list, device) -> tuple:
    """(f2, fgeos) tensors in the device layout from per-species arrays in
    Fortran order (NR,NT,NE,NPA) / (NT,NE,NPA), the same for every member."""
    g = gpu.grid
    f2 = np.zeros((gpu.n_members, gpu.ns, g.npa, g.ne, g.nt, g.nr))
    fg = np.zeros((gpu.n_members, gpu.ns, g.npa, g.ne, g.nt))
    for m in range(gpu.n_members):
        for s in range(gpu.ns):
            f2[m, s] = np.asarray(f2_list[s]).transpose(3, 2, 1, 0)
            fg[m, s] = np.asarray(fgeos_list[s]).transpose(2, 1, 0)
    return (torch.tensor(f2, device=device, requires_grad=True),
            torch.tensor(fg, device=device, requires_grad=True))
