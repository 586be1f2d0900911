"""torch.autograd.Function over the batched scorer (device pointers, no copies).

``UFFScore.apply(dofs, scorer)`` takes float32 CUDA tensors [B, 6 + nrb] in
the Optim.config layout (src/optim.ml:19-22) and returns the float64 energies
[B]; ``backward`` returns dE/d(dofs) from the hand-written adjoint kernels,
computed in the same launch sequence as the energies.  This is the torch entry
for Python scoring/optimisation scripts (the role of src/ff_score.py and
src/ff_opt.py in the reference, which call RDKit instead).
"""
from __future__ import annotations

import torch

from . import lib as _L
from .ff import UFFScorer


class UFFScore(torch.autograd.Function):
    @staticmethod
    def forward(ctx, dofs: torch.Tensor, scorer: UFFScorer, inter: bool = True,
                intra: bool = True, recenter: bool = False):
        if not dofs.is_cuda or dofs.dtype != torch.float32 or dofs.dim() != 2:
            raise ValueError("dofs must be a float32 CUDA tensor [B, 6 + nrb]")
        d = dofs.detach().contiguous()
        B, nd = d.shape
        if scorer.ligand is None or nd != 6 + scorer.ligand.nrb:
            raise ValueError("dofs must be [B, 6 + nrb] for the scorer's ligand")
        want_grad = dofs.requires_grad
        E = torch.empty(B, dtype=torch.float64, device=d.device)
        G = torch.empty((B, nd), dtype=torch.float32, device=d.device) if want_grad else None
        st = torch.empty(B, dtype=torch.int32, device=d.device)
        flags = ((_L.F_INTER if inter else 0) | (_L.F_INTRA if intra else 0) |
                 (_L.F_GRAD if want_grad else 0) | (_L.F_RECENTER if recenter else 0))
        stream = torch.cuda.current_stream(d.device).cuda_stream
        scorer.score_poses_device(d.data_ptr(), B, E.data_ptr(),
                                  G.data_ptr() if G is not None else None, st.data_ptr(),
                                  flags, stream)
        ctx.save_for_backward(G if G is not None else torch.empty(0, device=d.device))
        ctx.mark_non_differentiable(st)
        return E, st

    @staticmethod
    def backward(ctx, gE, _gst):
        (G,) = ctx.saved_tensors
        return (gE.to(torch.float32)[:, None] * G, None, None, None, None)


def uff_score(dofs: torch.Tensor, scorer: UFFScorer, inter=True, intra=True, recenter=False):
    """Energies [B] (float64) of a float32 [B, 6 + nrb] pose tensor."""
    E, _ = UFFScore.apply(dofs, scorer, inter, intra, recenter)
    return E
