"""Plain-PyTorch FP64 restatement of the macroscopic lookup, differentiable
with torch autograd -- the reference gradient for the GB300 adjoint.

It follows calculate_micro_xs / calculate_macro_xs
(openmp-threading/Simulation.c:241-375) with the interval of each nuclide
found by searchsorted, which on sorted energies is the same interval as the
unionized, nuclide and hash grids give (clamp(#{E_j <= E} - 1, 0, n_gp - 2)).
"""
from __future__ import annotations

import numpy as np
import torch


def tables_from_arrays(arrs: dict, n_iso: int, n_gp: int, max_nucs: int):
    """(egrid [n_iso, n_gp] numpy, xs [n_iso, n_gp, 5] float64 tensor,
    concs [12, max_nucs] tensor, mats [12, max_nucs] numpy, num_nucs) from
    HostProblem.arrays()."""
    grid = np.asarray(arrs["nuclide_grid"]).reshape(n_iso, n_gp, 6)
    egrid = np.ascontiguousarray(grid[:, :, 0])
    xs = torch.tensor(grid[:, :, 1:6].copy(), dtype=torch.float64)
    num_nucs = np.asarray(arrs["num_nucs"]).astype(int)
    mats = np.zeros((12, max_nucs), np.int64)
    concs = np.zeros((12, max_nucs), np.float64)
    o = 0
    for m in range(12):
        k = num_nucs[m]
        mats[m, :k] = arrs["mats"][o:o + k]
        concs[m, :k] = arrs["concs"][o:o + k]
        o += k
    return egrid, xs, torch.tensor(concs), mats, num_nucs


def macro_xs(E, mat, concs, xs, egrid, mats, num_nucs):
    """macro_xs [n, 5] for energies E (tensor, may require grad) and materials
    mat (numpy int)."""
    n = E.shape[0]
    n_gp = egrid.shape[1]
    out = torch.zeros((n, 5), dtype=torch.float64)
    e_np = E.detach().numpy()
    # one view per nuclide: the backward of each gather is then one nuclide's
    # [n_gp, 5] block instead of a dense copy of the whole table
    xs_n = xs.unbind(0)
    for m in range(12):
        rows = np.nonzero(mat == m)[0]
        if rows.size == 0:
            continue
        idx = torch.from_numpy(rows)
        Em = E[idx]
        for j in range(num_nucs[m]):
            nuc = int(mats[m, j])
            k = np.searchsorted(egrid[nuc], e_np[rows], side="right") - 1
            k = np.clip(k, 0, n_gp - 2)
            kt = torch.from_numpy(k)
            lo_e = torch.from_numpy(egrid[nuc][k])
            hi_e = torch.from_numpy(egrid[nuc][k + 1])
            f = (hi_e - Em) / (hi_e - lo_e)
            lo = xs_n[nuc][kt]
            hi = xs_n[nuc][kt + 1]
            micro = hi - f[:, None] * (hi - lo)
            out = out.index_add(0, idx, micro * concs[m, j])
    return out


def reference_gradients(E_np, mat_np, gbar_np, egrid, xs, concs, mats, num_nucs):
    """(macro, dL/dE, dL/dconcs, dL/dxs) for L = sum(gbar * macro_xs)."""
    E = torch.tensor(E_np, dtype=torch.float64, requires_grad=True)
    c = concs.clone().requires_grad_(True)
    x = xs.clone().requires_grad_(True)
    macro = macro_xs(E, mat_np, c, x, egrid, mats, num_nucs)
    L = (torch.tensor(gbar_np) * macro).sum()
    dE, dc, dx = torch.autograd.grad(L, [E, c, x])
    return macro.detach().numpy(), dE.numpy(), dc.numpy(), dx.numpy()
