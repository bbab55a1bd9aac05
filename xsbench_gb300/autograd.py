"""A thin torch.autograd.Function over the C-ABI lookup and its adjoint.

For checking gradients with torch's tools only: the forward runs
``xs_lookup_samples`` and the backward ``xs_adjoint_samples`` on a context
(Context).  The concentration and cross-section tensors passed in are the
autograd leaves that stand for the context's own tables (their values are
not read: the context holds the tables); their gradients come back in the
layouts concs[12, max_num_nucs] and xs[n_isotopes, n_gridpoints, 5]
(channels total, elastic, absorbtion, fission, nu_fission).
"""
from __future__ import annotations

import torch


class MacroXS(torch.autograd.Function):
    @staticmethod
    def forward(fctx, energy, mat, concs, xs, xsctx):
        n = energy.shape[0]
        macro = torch.empty((n, 5), dtype=torch.float64, device=energy.device)
        xsctx.lookup_samples(energy.contiguous(), mat.contiguous(), macro_out=macro)
        fctx.save_for_backward(energy, mat)
        fctx.xsctx = xsctx
        fctx.shapes = (concs.shape, xs.shape)
        return macro

    @staticmethod
    def backward(fctx, gbar):
        energy, mat = fctx.saved_tensors
        cshape, xshape = fctx.shapes
        d_e = torch.empty_like(energy)
        d_c = torch.zeros(cshape, dtype=torch.float64, device=energy.device)
        d_x = torch.zeros(xshape, dtype=torch.float64, device=energy.device)
        fctx.xsctx.adjoint(gbar.contiguous(), energy=energy.contiguous(), mat=mat.contiguous(),
                           d_concs=d_c, d_xs=d_x, d_energy=d_e)
        return d_e, None, d_c, d_x, None


def macro_xs(energy, mat, concs, xs, xsctx):
    return MacroXS.apply(energy, mat, concs, xs, xsctx)
