"""The adjoint of the lookup (xs_run_adjoint / xs_adjoint_samples).

Bars: every gradient array within 1e-8 relative (max norm over the array,
max|a - b| / max|b|) of the plain-PyTorch FP64 reference gradient
(tests/torch_reference.py) and of central finite differences (h = 1e-6) of
the oracle's forward; bit-identical results on repeated runs.  Sizes: 68
nuclides x 1000 gridpoints, 100,000 lookups; the forward + adjoint
configuration of the benchmark (68 nuclides x 11,303 gridpoints, 100,000
lookups, all three grids) against both; the full-size problem (355 x 11,303,
17M lookups, unionized grid with its union table and hash grid) on 20,000
lookups spread over the batch, and through linearity (the gradient of a split
batch adds up).
"""
import numpy as np
import pytest

import oracle
import xsbench_gb300 as X
from conftest import oracle_config, product_inputs
from torch_reference import macro_xs, reference_gradients, tables_from_arrays

N = 100000
TOL = 1e-8


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def rel_rows(a, b):
    """Largest per-lookup relative difference of macro_xs vectors (max norm)."""
    num = np.max(np.abs(a - b), axis=1)
    return float(np.max(num / np.maximum(np.max(np.abs(b), axis=1), 1e-300)))


def fd_tol(ad, lp, lm, h):
    """Tolerance of a central difference: the 1e-8 bar plus the rounding of
    the two functional values (their ulps divided by 2h)."""
    return TOL * max(abs(ad), 1.0) + 4e-16 * (abs(lp) + abs(lm)) / (2 * h)


def gbar_for(n, seed=1234):
    return np.random.default_rng(seed).standard_normal((n, 5))


@pytest.fixture(scope="module")
def tiny_problem():
    inp = product_inputs("tiny_unionized")
    with X.grid_init(inp) as p:
        arrs = {k: np.array(v) for k, v in p.arrays().items()}
    return inp, arrs


def test_torch_reference_forward_matches_oracle(tiny_problem):
    """The torch restatement reproduces the oracle's macro_xs (CPU)."""
    import torch
    inp, arrs = tiny_problem
    egrid, xs, concs, mats, nn = tables_from_arrays(arrs, 68, 1000, 34)
    with oracle.Problem(oracle_config("tiny_unionized")) as o:
        r = o.run_event(n=20000, want_macro=True, want_samples=True)
    out = macro_xs(torch.tensor(r["energy"]), r["mat"], concs, xs, egrid, mats, nn).numpy()
    num = np.max(np.abs(out - r["macro"]), axis=1)
    assert np.max(num / np.max(np.abs(r["macro"]), axis=1)) <= 1e-13


@pytest.fixture(scope="module")
def ctxs(tiny_problem):
    out = {}
    yield out
    for prob, ctx in out.values():
        ctx.close()
        prob.close()


def ctx_for(ctxs, name):
    if name not in ctxs:
        inp = product_inputs(name)
        prob = X.grid_init(inp)
        ctxs[name] = (prob, X.Context(inp, prob))
    return ctxs[name]


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["tiny_unionized", "tiny_hash", "tiny_nuclide"])
def test_adjoint_against_torch_reference(ctxs, name):
    prob, ctx = ctx_for(ctxs, name)
    arrs = prob.arrays()
    egrid, xs, concs, mats, nn = tables_from_arrays(arrs, 68, 1000, 34)
    g = gbar_for(N)
    macro = np.empty((N, 5))
    d_e = np.empty(N)
    d_c = np.zeros((12, 34))
    d_x = np.zeros((68, 1000, 5))
    r = ctx.adjoint(g, count=N, macro_out=macro, d_concs=d_c, d_xs=d_x, d_energy=d_e)
    E, M = ctx.sample_event(0, N)
    ref_macro, ref_e, ref_c, ref_x = reference_gradients(E, M, g, egrid, xs, concs, mats, nn)
    assert rel(macro, ref_macro) <= 1e-12
    assert rel(d_e, ref_e) <= TOL
    assert rel(d_c, ref_c) <= TOL
    assert rel(d_x, ref_x) <= TOL
    assert r.verification == ctx.run_event(count=N).verification
    assert r.kernel_launches >= 8


@pytest.mark.gpu
def test_adjoint_is_bit_reproducible_and_host_device_agree(ctxs):
    import torch
    prob, ctx = ctx_for(ctxs, "tiny_unionized")
    g = gbar_for(N, seed=7)
    outs = []
    for _ in range(2):
        d_e = np.empty(N)
        d_c = np.zeros((12, 34))
        d_x = np.zeros((68, 1000, 5))
        ctx.adjoint(g, count=N, d_concs=d_c, d_xs=d_x, d_energy=d_e)
        outs.append((d_e, d_c, d_x))
    for a, b in zip(*outs):
        assert np.array_equal(a, b)
    dg = torch.from_numpy(g).cuda()
    dd_e = torch.empty(N, dtype=torch.float64, device="cuda")
    dd_c = torch.zeros((12, 34), dtype=torch.float64, device="cuda")
    dd_x = torch.zeros((68, 1000, 5), dtype=torch.float64, device="cuda")
    ctx.adjoint(dg, count=N, d_concs=dd_c, d_xs=dd_x, d_energy=dd_e)
    torch.cuda.synchronize()
    assert np.array_equal(dd_e.cpu().numpy(), outs[0][0])
    assert np.array_equal(dd_c.cpu().numpy(), outs[0][1])
    assert np.array_equal(dd_x.cpu().numpy(), outs[0][2])


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["tiny_unionized", "tiny_hash"])
def test_adjoint_repeated_energies(ctxs, name):
    """Caller samples with repeated energies, which exercise every path of the
    per-bucket sort: 40 distinct energies over most lookups (buckets whose
    keys crowd one range: the shared-memory network), 3,000 fuel lookups at
    one energy (a bucket above the shared-memory capacity: the in-place
    network), the rest distinct (the range sort).  Against the torch
    reference, and bit-identical on a second run."""
    prob, ctx = ctx_for(ctxs, name)
    egrid, xs, concs, mats, nn = tables_from_arrays(prob.arrays(), 68, 1000, 34)
    n = 60000
    E, M = ctx.sample_event(0, n)
    rng = np.random.default_rng(21)
    E = E.copy()
    M = M.copy()
    E[:40000] = rng.random(40)[rng.integers(0, 40, 40000)]
    E[40000:43000] = 0.4375
    M[40000:43000] = 0
    g = gbar_for(n, seed=9)
    outs = []
    for _ in range(2):
        macro = np.empty((n, 5))
        d_e = np.empty(n)
        d_c = np.zeros((12, 34))
        d_x = np.zeros((68, 1000, 5))
        ctx.adjoint(g, energy=E, mat=M, macro_out=macro, d_concs=d_c, d_xs=d_x, d_energy=d_e)
        outs.append((macro, d_e, d_c, d_x))
    for a, b in zip(*outs):
        assert np.array_equal(a, b)
    ref_macro, ref_e, ref_c, ref_x = reference_gradients(E, M, g, egrid, xs, concs, mats, nn)
    macro, d_e, d_c, d_x = outs[0]
    assert rel(macro, ref_macro) <= 1e-12
    assert rel(d_e, ref_e) <= TOL
    assert rel(d_c, ref_c) <= TOL
    assert rel(d_x, ref_x) <= TOL


def check_central_differences(ctx, name, n_gp, max_nucs, n, d_c, d_x, d_e, g, E, M):
    """Central differences (h = 1e-6) of the oracle's forward on per-lookup
    functionals against the adjoint's d_concs, d_xs and d_energy of lookups
    (E, M) with upstream gradients g."""
    h = 1e-6
    with oracle.Problem(oracle_config(name)) as o:
        egrid = o.arrays()["nuclide_grid"].reshape(68, n_gp, 6)[:, :, 0]

        def L(sel, energies=None):
            e = E[sel] if energies is None else energies
            r = o.run_samples(e, M[sel], nthreads=1)
            return float(np.sum(g[sel] * r["macro"]))

        # concentrations: L is linear in them, so FD is exact up to rounding
        for m, j in ((0, 0), (0, 33), (2, 1), (4, 26), (11, 8)):
            sel = np.nonzero(M == m)[0]
            p = o.sd.concs
            idx = m * max_nucs + j
            c0 = p[idx]
            p[idx] = c0 + h
            lp = L(sel)
            p[idx] = c0 - h
            lm = L(sel)
            p[idx] = c0
            fd = (lp - lm) / (2 * h)
            assert abs(fd - d_c[m, j]) <= fd_tol(d_c[m, j], lp, lm, h), (m, j, fd, d_c[m, j])

        # tabulated xs: restrict L to the lookups near the perturbed gridpoint
        grid = o.sd.nuclide_grid
        for nuc, pt, ch in ((58, n_gp // 2, 0), (24, 10, 3), (63, n_gp - 2, 4), (41, 1, 1)):
            lo_e = egrid[nuc][max(pt - 1, 0)]
            hi_e = egrid[nuc][min(pt + 1, n_gp - 1)]
            sel = np.nonzero((E >= lo_e) & (E <= hi_e))[0]
            if pt <= 1:
                sel = np.nonzero(E <= hi_e)[0]
            if pt >= n_gp - 2:
                sel = np.nonzero(E >= lo_e)[0]
            field = ("total_xs", "elastic_xs", "absorbtion_xs", "fission_xs", "nu_fission_xs")[ch]
            gp = grid[nuc * n_gp + pt]
            v0 = getattr(gp, field)
            setattr(grid[nuc * n_gp + pt], field, v0 + h)
            lp = L(sel)
            setattr(grid[nuc * n_gp + pt], field, v0 - h)
            lm = L(sel)
            setattr(grid[nuc * n_gp + pt], field, v0)
            fd = (lp - lm) / (2 * h)
            assert abs(fd - d_x[nuc, pt, ch]) <= fd_tol(d_x[nuc, pt, ch], lp, lm, h), (nuc, pt, ch)

        # energy: lookups whose [E-h, E+h] stays inside every bracket
        arrs = o.arrays()
        offs = np.concatenate([[0], np.cumsum(arrs["num_nucs"])])
        checked = 0
        for i in range(n):
            m = M[i]
            nucs = arrs["mats"][offs[m]:offs[m + 1]]
            ok = all(np.searchsorted(egrid[nu], E[i] - h, "right") == np.searchsorted(egrid[nu], E[i] + h, "right")
                     for nu in nucs)
            if not ok:
                continue
            sel = np.array([i])
            lp = L(sel, np.array([E[i] + h]))
            lm = L(sel, np.array([E[i] - h]))
            fd = (lp - lm) / (2 * h)
            assert abs(fd - d_e[i]) <= fd_tol(d_e[i], lp, lm, h), (i, fd, d_e[i])
            checked += 1
            if checked == 40:
                break
        assert checked == 40


@pytest.mark.gpu
def test_adjoint_against_central_differences(ctxs):
    """FD (h = 1e-6) of the oracle's forward, on per-lookup functionals."""
    prob, ctx = ctx_for(ctxs, "tiny_unionized")
    n = 20000
    g = gbar_for(n, seed=11)
    d_e = np.empty(n)
    d_c = np.zeros((12, 34))
    d_x = np.zeros((68, 1000, 5))
    ctx.adjoint(g, count=n, d_concs=d_c, d_xs=d_x, d_energy=d_e)
    E, M = ctx.sample_event(0, n)
    check_central_differences(ctx, "tiny_unionized", 1000, 34, n, d_c, d_x, d_e, g, E, M)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["small_unionized", "small_hash", "small_nuclide"])
def test_adjoint_benchmark_configuration_small(name):
    """The forward + adjoint configuration at the size its check is defined
    for: 68 nuclides x 11,303 gridpoints, 100,000 lookups of the event batch,
    upstream gradients N(0,1); every gradient array and macro_xs against the
    plain-PyTorch FP64 reference (1e-8 / 1e-12), and central differences of
    the oracle's forward (h = 1e-6, bracket-safe energies)."""
    inp = product_inputs(name)
    n, n_gp = N, 11303
    with X.grid_init(inp) as prob, X.Context(inp, prob) as ctx:
        g = gbar_for(n, seed=29)
        macro = np.empty((n, 5))
        d_e = np.empty(n)
        d_c = np.zeros((12, 34))
        d_x = np.zeros((68, n_gp, 5))
        r = ctx.adjoint(g, count=n, macro_out=macro, d_concs=d_c, d_xs=d_x, d_energy=d_e)
        assert r.verification == ctx.run_event(count=n).verification
        E, M = ctx.sample_event(0, n)
        egrid, xs, concs, mats, nn = tables_from_arrays(prob.arrays(), 68, n_gp, 34)
    ref_macro, ref_e, ref_c, ref_x = reference_gradients(E, M, g, egrid, xs, concs, mats, nn)
    assert rel_rows(macro, ref_macro) <= 1e-12
    assert rel(d_e, ref_e) <= TOL
    assert rel(d_c, ref_c) <= TOL
    assert rel(d_x, ref_x) <= TOL
    check_central_differences(None, name, n_gp, 34, n, d_c, d_x, d_e, g, E, M)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["large_unionized", "large_hash"])
def test_adjoint_full_size_against_torch_reference(name):
    """The benchmarked forward + adjoint at full size: 355 nuclides x 11,303
    gridpoints, 17M lookups.  On the unionized grid the context builds its
    union table, and the adjoint's forward pass reads it, which is the path
    the benchmark times.  (1) The whole batch through xs_run_adjoint on
    device arrays: macro_xs and the energy gradient (per-lookup values) of
    20,000 lookups spread over the batch against the torch reference.  (2)
    Those 20,000 lookups as caller samples through xs_adjoint_samples (the
    same kernels): all three gradient arrays against the torch reference."""
    import torch
    inp = product_inputs(name)
    n_gp, mx = 11303, 321
    with X.grid_init(inp) as p, X.Context(inp, p) as ctx:
        if name == "large_unionized":
            assert ctx.union_table_bytes > 0
        n = inp.lookups
        g = gbar_for(n, seed=17)
        dev = dict(dtype=torch.float64, device="cuda")
        d_e, macro = torch.empty(n, **dev), torch.empty((n, 5), **dev)
        d_c, d_x = torch.zeros((12, mx), **dev), torch.zeros((355, n_gp, 5), **dev)
        r = ctx.adjoint(torch.from_numpy(g).cuda(), macro_out=macro, d_concs=d_c, d_xs=d_x,
                        d_energy=d_e)
        assert r.hash == X.EXPECTED_HASH[("event", "large")]
        sel = np.linspace(0, n - 1, 20000).astype(np.int64)
        d_e_sel = d_e.cpu().numpy()[sel]
        macro_sel = macro.cpu().numpy()[sel]
        del d_e, macro, d_c, d_x
        E, M = ctx.sample_event(0, n)
        Es, Ms, gs = E[sel].copy(), M[sel].copy(), np.ascontiguousarray(g[sel])
        del E, M, g
        m2, e2 = np.empty((sel.size, 5)), np.empty(sel.size)
        c2, x2 = np.zeros((12, mx)), np.zeros((355, n_gp, 5))
        ctx.adjoint(gs, energy=Es, mat=Ms, macro_out=m2, d_concs=c2, d_xs=x2, d_energy=e2)
        egrid, xs, concs, mats, nn = tables_from_arrays(p.arrays(), 355, n_gp, mx)
    ref_macro, ref_e, ref_c, ref_x = reference_gradients(Es, Ms, gs, egrid, xs, concs, mats, nn)
    assert rel_rows(macro_sel, ref_macro) <= 1e-12
    assert rel(d_e_sel, ref_e) <= TOL
    assert rel_rows(m2, ref_macro) <= 1e-12
    assert rel(e2, ref_e) <= TOL
    assert rel(c2, ref_c) <= TOL
    assert rel(x2, ref_x) <= TOL


@pytest.mark.gpu
def test_autograd_function_matches_torch_reference(ctxs):
    import torch
    from xsbench_gb300.autograd import macro_xs as gpu_macro
    prob, ctx = ctx_for(ctxs, "tiny_hash")
    egrid, xs, concs, mats, nn = tables_from_arrays(prob.arrays(), 68, 1000, 34)
    n = 30000
    E, M = ctx.sample_event(0, n)
    g = gbar_for(n, seed=5)
    dE_t = torch.tensor(E, device="cuda", requires_grad=True)
    c_t = concs.cuda().requires_grad_(True)
    x_t = xs.cuda().requires_grad_(True)
    out = gpu_macro(dE_t, torch.tensor(M, device="cuda"), c_t, x_t, ctx)
    L = (torch.tensor(g, device="cuda") * out).sum()
    ge, gc, gx = torch.autograd.grad(L, [dE_t, c_t, x_t])
    ref = reference_gradients(E, M, g, egrid, xs, concs, mats, nn)
    assert rel(out.detach().cpu().numpy(), ref[0]) <= 1e-12
    assert rel(ge.cpu().numpy(), ref[1]) <= TOL
    assert rel(gc.cpu().numpy(), ref[2]) <= TOL
    assert rel(gx.cpu().numpy(), ref[3]) <= TOL


@pytest.mark.gpu
def test_adjoint_full_size_linearity():
    """Large hash grid, 17M lookups: the gradient sums of the whole batch equal
    those of its two halves (size-independent property), and the energy
    gradient of sampled lookups matches the torch reference."""
    inp = product_inputs("large_hash")
    with X.grid_init(inp) as p, X.Context(inp, p) as ctx:
        n = inp.lookups
        g = gbar_for(n, seed=3)
        shape_c, shape_x = (12, 321), (355, 11303, 5)
        d_e = np.empty(n)
        c_all, x_all = np.zeros(shape_c), np.zeros(shape_x)
        r = ctx.adjoint(g, d_concs=c_all, d_xs=x_all, d_energy=d_e)
        assert r.hash == X.EXPECTED_HASH[("event", "large")]
        c_half, x_half = np.zeros(shape_c), np.zeros(shape_x)
        h = n // 2
        ctx.adjoint(np.ascontiguousarray(g[:h]), first=0, count=h, d_concs=c_half, d_xs=x_half)
        ctx.adjoint(np.ascontiguousarray(g[h:]), first=h, count=n - h, d_concs=c_half, d_xs=x_half)
        assert rel(c_half, c_all) <= 1e-10
        assert rel(x_half, x_all) <= 1e-10
        sel = np.arange(0, n, n // 997)[:997]
        E, M = ctx.sample_event(0, n)
        egrid, xs, concs, mats, nn = tables_from_arrays(p.arrays(), 355, 11303, 321)
        ref = reference_gradients(E[sel], M[sel], g[sel], egrid, xs, concs, mats, nn)
        assert rel(d_e[sel], ref[1]) <= TOL
