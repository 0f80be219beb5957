"""Thin torch binding of the personalised-PageRank C ABI for tests: a
torch.autograd.Function whose forward is gbx_ppr_forward and whose backward
is the hand-written adjoint gbx_ppr_adjoint, called with the upstream
gradient dL/dR as the adjoint's loss weights. Not part of the library."""
from __future__ import annotations

import torch

from graphblox_gb300 import graph as gg


class PersonalisedPageRank(torch.autograd.Function):
    @staticmethod
    def forward(ctx, weights, teleport, dg, damping=0.85, tol=1e-7, max_iterations=1000):
        weights = weights.detach().contiguous()
        teleport = teleport.detach().contiguous()
        st = gg.ppr_forward(dg, weights, teleport, damping, tol, max_iterations)
        ctx.dg, ctx.damping, ctx.tol, ctx.max_iterations = dg, damping, tol, max_iterations
        ctx.iterations = st.iterations
        ctx.save_for_backward(weights, st.ranks)
        return st.ranks

    @staticmethod
    def backward(ctx, grad_ranks):
        weights, ranks = ctx.saved_tensors
        adj = gg.ppr_adjoint(ctx.dg, weights, ranks, grad_ranks.contiguous(), ctx.damping, ctx.tol,
                             ctx.max_iterations, want_weights=ctx.needs_input_grad[0],
                             want_teleport=ctx.needs_input_grad[1])
        return adj.grad_weights, adj.grad_teleport, None, None, None, None


def personalised_pagerank(weights, teleport, dg, damping=0.85, tol=1e-7, max_iterations=1000):
    return PersonalisedPageRank.apply(weights, teleport, dg, damping, tol, max_iterations)
