"""torch.autograd bindings of the hand-written adjoints (the Python
counterpart of a ChainRulesCore rrule).

``BPEnergy.apply(tn, terms, update_kwargs, *tensors)`` runs BP to convergence
on the GPU, returns the BP energy sum_e <h_e>, and in backward returns
dE/dA_v through the fixed point by implicit differentiation (the adjoint BP
solve); nothing is recorded on torch's tape between the two."""
from __future__ import annotations

import numpy as np
import torch

from .cache import BeliefPropagationCache


class BPEnergy(torch.autograd.Function):
    @staticmethod
    def forward(ctx, tn, terms, update_kwargs, *tensors):
        net = tn.copy()
        net.tensors = [t.detach().cpu().double().numpy() for t in tensors]
        bpc = BeliefPropagationCache(net)
        bpc.update(**(update_kwargs or {}))
        energy, grad = bpc.energy2_grad(terms, mode="implicit")
        bpc.close()
        ctx.grads = [torch.from_numpy(np.asarray(g)).to(tensors[i].dtype) for i, g in enumerate(grad)]
        return torch.tensor(float(energy), dtype=torch.float64)

    @staticmethod
    def backward(ctx, gout):
        return (None, None, None, *[gout.to(g.dtype) * g for g in ctx.grads])
