"""The batched kernel finds hash-grid intervals with a warp-cooperative search
for the bracketing interval and applies the hash lookup's edge rule only
where it can differ.  This checks that rule against the reference's hash
search (openmp-threading/Simulation.c:273-301) for every (lookup, nuclide)
pair of the 68-nuclide, 500-bin problem and for energies placed on gridpoints
and bin edges, on the CPU (numpy over the oracle's setup arrays)."""
import numpy as np

import oracle
from conftest import oracle_config


def reference_hash_interval(g, idx_row_lo, idx_row_hi, last_bin, E):
    """Simulation.c:273-301 for one nuclide's energies g, vectorised over E."""
    n = g.shape[0]
    u_low = idx_row_lo
    u_high = np.where(last_bin, n - 1, idx_row_hi + 1)
    e_low, e_high = g[u_low], g[u_high]
    # grid_search_nuclide over [u_low, u_high]: largest i in [u_low, u_high-1] with g[i] <= E
    inner = np.clip(np.searchsorted(g, E, side="right") - 1, u_low, u_high - 1)
    lower = np.where(E <= e_low, 0, np.where(E >= e_high, n - 1, inner))
    return np.where(lower == n - 1, lower - 1, lower)


def kernel_rule(g, idx_lo, idx_hi, last_bin, b, du, E):
    """The batched kernel's rule: the bracketing interval, the edge rule when E
    equals the gridpoint below, the reference search when E / du put E
    outside [b*du, (b+1)*du)."""
    n = g.shape[0]
    cnt = np.searchsorted(g, E, side="right")
    k = np.clip(cnt - 1, 0, n - 2)
    eq = (cnt > 0) & (g[np.maximum(cnt - 1, 0)] == E)
    edge = eq & (k > 0) & (E <= g[idx_lo])
    k = np.where(edge, 0, k)
    outside = (b * du > E) | (~last_bin & ((b + 1) * du <= E))
    ref = reference_hash_interval(g, idx_lo, idx_hi, last_bin, E)
    return np.where(outside, ref, k)


def test_kernel_hash_rule_matches_reference():
    name = "tiny_hash"
    with oracle.Problem(oracle_config(name)) as o:
        a = {k: np.array(v) for k, v in o.arrays().items()}
        r = o.run_event(want_samples=True)
    n_iso, n_gp, bins = 68, 1000, 500
    grid = a["nuclide_grid"].reshape(n_iso, n_gp, 6)[:, :, 0]
    index = a["index_grid"].reshape(bins, n_iso)
    du = 1.0 / bins
    rng = np.random.default_rng(7)
    # the sampled lookups, plus energies on gridpoints and on / next to bin edges
    extra = [grid.ravel()[rng.integers(0, grid.size, 4000)],
             np.arange(bins) * du,
             np.nextafter(np.arange(1, bins) * du, 0.0),
             np.nextafter(np.arange(bins) * du, 1.0)]
    E_all = np.concatenate([r["energy"], *extra])
    checked = 0
    for nuc in range(n_iso):
        g = grid[nuc]
        E = E_all
        b = np.clip((E / du).astype(np.int64), 0, bins - 1)
        last = b == bins - 1
        lo = index[b, nuc]
        hi = index[np.minimum(b + 1, bins - 1), nuc]
        ref = reference_hash_interval(g, lo, hi, last, E)
        got = kernel_rule(g, lo, hi, last, b, du, E)
        assert np.array_equal(ref, got), nuc
        checked += E.size
    assert checked > 10_000_000


def guided_rule(g, guide, K, E, certain, ref):
    """The plain kernel's guided search (macro_xs_guided): start at
    clamp(guide[floor(E 2^K)] - 1, 0, n - 2), step up while E >= the
    interval's upper energy; on the hash grid, `ref` where E is not certainly
    inside its hash bin or equals the interval's lower gridpoint."""
    n = g.shape[0]
    b = np.floor(E * 2.0 ** K).astype(np.int64)
    k = np.clip(guide[b] - 1, 0, n - 2)
    while True:
        step = (k < n - 2) & ~(E < g[np.minimum(k + 1, n - 1)])
        if not step.any():
            break
        k = k + step
    if certain is None:
        return k
    return np.where(~certain | (g[k] == E), ref, k)


def test_guided_search_matches_reference():
    """The guided search gives the reference's interval on the hash grid
    (Simulation.c:273-301) and on the nuclide grid (:252-263) for the sampled
    lookups and for energies on gridpoints, on and next to hash bin edges,
    next to guide bin edges, and at 0."""
    with oracle.Problem(oracle_config("tiny_hash")) as o:
        a = {k: np.array(v) for k, v in o.arrays().items()}
        r = o.run_event(want_samples=True)
    n_iso, n_gp, bins = 68, 1000, 500
    grid = a["nuclide_grid"].reshape(n_iso, n_gp, 6)[:, :, 0]
    index = a["index_grid"].reshape(bins, n_iso)
    du = 1.0 / bins
    K = 12   # the guide size the context picks for 1,000 gridpoints: 2^(10 + 2) bins
    rng = np.random.default_rng(11)
    edges_k = np.arange(1, 2 ** K) / 2.0 ** K
    extra = [grid.ravel()[rng.integers(0, grid.size, 4000)],
             np.arange(bins) * du, np.nextafter(np.arange(1, bins) * du, 0.0),
             np.nextafter(np.arange(bins) * du, 1.0), edges_k, np.nextafter(edges_k, 0.0),
             np.array([0.0, np.nextafter(0.0, 1.0), np.nextafter(1.0, 0.0)])]
    E = np.concatenate([r["energy"], *extra])
    # xsgb_hash_bin's certainty: E * bins more than bins * 2^-50 from an integer
    x = E.astype(np.longdouble) * bins
    certain = (np.abs(x - np.rint(x)) > bins * 2.0 ** -50) & (E > 0)
    b = np.clip((E / du).astype(np.int64), 0, bins - 1)
    last = b == bins - 1
    for nuc in range(n_iso):
        g = grid[nuc]
        guide = np.searchsorted(g, np.arange(2 ** K + 1) / 2.0 ** K, side="left")
        ref_h = reference_hash_interval(g, index[b, nuc], index[np.minimum(b + 1, bins - 1), nuc],
                                        last, E)
        assert np.array_equal(guided_rule(g, guide, K, E, certain, ref_h), ref_h), nuc
        ref_n = np.clip(np.searchsorted(g, E, side="right") - 1, 0, n_gp - 2)
        assert np.array_equal(guided_rule(g, guide, K, E, None, None), ref_n), nuc
