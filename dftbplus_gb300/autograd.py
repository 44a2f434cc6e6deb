"""Differentiable SCC-DFTB energy for PyTorch over the C-ABI.

``DftbEnergy(model, species)(coords, sk_ham, sk_over, hubbu)`` returns the converged Mermin free
energy as a 0-d float64 tensor; ``backward`` gives dE/dcoords (the gradient kernel, the force
contraction of forces.F90:548-669), dE/d(SK grid values) of the H and S tables in the packed table
layout of ``Model.pack()``, and dE/dU per species (``dftbgpu_grad_params``). All derivatives are the
hand-written adjoints of the library: at SCC convergence the energy is stationary in the density
matrix and the charges, so no derivative of the iterations is needed. Mirrors the call pattern of
the reference's Python API (tools/pythonapi/src/dftbplus/dftbplus.py: get_energy, get_gradients).
"""
from __future__ import annotations

import numpy as np
import torch

from . import binding
from .model import Model


class _DftbFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, coords, sk_ham, sk_over, hubbu, eng):
        p = dict(eng.base)
        p["sk_ham"] = sk_ham.detach().cpu().numpy().astype(np.float64)
        p["sk_over"] = sk_over.detach().cpu().numpy().astype(np.float64)
        p["hubbu"] = hubbu.detach().cpu().numpy().astype(np.float64)
        eng.ctx.set_model_packed(p)
        eng.ctx.set_geometry(coords.detach().cpu().numpy(), eng.species)
        res = eng.ctx.scc(eng.opts)
        if not res["converged"]:
            raise binding.DftbGpuError(4, "SCC is NOT converged; the variational derivatives do not apply")
        g = eng.ctx.gradients()
        gh, go, gu = eng.ctx.grad_params()
        ctx.save_for_backward(torch.from_numpy(g).to(coords), torch.from_numpy(gh).to(sk_ham),
                              torch.from_numpy(go).to(sk_over), torch.from_numpy(gu).to(hubbu))
        eng.last = res
        return torch.tensor(res["energies"]["EMermin"], dtype=torch.float64, device=coords.device)

    @staticmethod
    def backward(ctx, grad_e):
        g, gh, go, gu = ctx.saved_tensors
        return grad_e * g, grad_e * gh, grad_e * go, grad_e * gu, None


class DftbEnergy:
    """Energy functional E(coords, SK tables, U) of one system (species fixed) on one GB300."""

    def __init__(self, model: Model, species, kT: float = 1e-3, scc_tol: float = 1e-9, device: int = 0):
        self.model = model
        self.species = np.asarray(species, dtype=np.int32)
        self.base = model.pack()
        self.ctx = binding.Context(device)
        self.opts = binding.default_opts(kT=kT, scc_tol=scc_tol)
        self.last = None

    def parameters(self):
        """Initial parameter tensors (float64): sk_ham, sk_over (packed layout), hubbu."""
        return (torch.tensor(self.base["sk_ham"], dtype=torch.float64),
                torch.tensor(self.base["sk_over"], dtype=torch.float64),
                torch.tensor(self.base["hubbu"], dtype=torch.float64))

    def __call__(self, coords, sk_ham, sk_over, hubbu):
        return _DftbFunction.apply(coords, sk_ham, sk_over, hubbu, self)

    def close(self):
        self.ctx.close()
