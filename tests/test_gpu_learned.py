"""The learned preconditioner end to end (no reference counterpart): a linear U-Net
trained on the GPU by the library's own kernels on 32^3 (f, u) pairs solved by the
plain FP64 solver, used as the coarse-grid solver inside flexible CG; it must cut the
iteration count of the method without it and still meet the FP64 tolerance, and an
untrained network must trigger the fallback to the plain preconditioner."""
import math

import numpy as np
import pytest

import parallelpoissonsolver_gb300 as pps
from parallelpoissonsolver_gb300 import learned
from conftest import rel_l2

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

FLAGS = pps.LEARNED_INITIAL_GUESS | pps.LEARNED_PRECONDITIONER | pps.LEARNED_POST_SMOOTH


@pytest.fixture(scope="module")
def trained(gpu):
    train = learned.make_dataset(32, range(10000, 10128))
    held = learned.make_dataset(32, range(30000, 30004))
    scale = learned.fit_scale(train)
    net = pps.UNet((16, 32, 64), seed=1, linear=True)
    losses = learned.train(net, train, scale, 2500, lr=1e-3)
    errs = learned.evaluate(net, held, scale)
    yield net, scale, losses, errs
    net.close()


def gain_for(m, scale):
    k = int(round(math.log2(m / 32)))
    return k, scale * ((2 ** k / (m + 1)) / (1.0 / 33)) ** 2


def test_training_reaches_a_useful_network(trained):
    net, scale, losses, errs = trained
    assert np.mean(losses[-100:]) < 0.1 * np.mean(losses[:100])
    assert max(errs) < 0.15, errs


@pytest.mark.parametrize("form", ["fp64", "mixed"])
def test_learned_preconditioner_cuts_iterations(trained, oracle, form):
    net, scale, _, _ = trained
    m = 64
    grid = pps.BlockGrid.cube(m)
    k, gain = gain_for(m, scale)
    b = learned.rhs(m, 30010, "field")
    x_ref = np.zeros_like(b)
    oracle.solve(oracle.cube(m), oracle.Config(tol=1e-13, maxit=20000, threads=4), x_ref, b.copy())
    plain = pps.FlexibleCG(grid, pps.ChebyshevIteration(11), tolerance=1e-10, form=form)
    x0 = np.zeros_like(b)
    assert plain(x0, b.copy()) == pps.OK
    it_plain = plain.get_num_iteration_final()
    s = pps.FlexibleCG(grid, pps.ChebyshevIteration(11), tolerance=1e-10, form=form, use_graph=False)
    s.set_learned(net, k, gain, FLAGS)
    x = np.zeros_like(b)
    assert s(x, b.copy()) == pps.OK
    st = s.stats()
    assert st["fallback_iteration"] == -1 and st["learned_applications"] > 0
    assert s.get_error_compute_operator() <= 1e-10
    assert s.get_num_iteration_final() <= 0.5 * it_plain, (s.get_num_iteration_final(), it_plain)
    assert rel_l2(x, x_ref) < 1e-6


def test_untrained_network_falls_back(gpu, oracle):
    net = pps.UNet((16, 32, 64), seed=5)                 # random weights
    m = 64
    grid = pps.BlockGrid.cube(m)
    b = learned.rhs(m, 30011, "blobs")
    s = pps.FlexibleCG(grid, pps.ChebyshevIteration(11), tolerance=1e-10, form="fp64", use_graph=False)
    s.set_learned(net, 1, 1e-3, pps.LEARNED_PRECONDITIONER)
    x = np.zeros_like(b)
    assert s(x, b.copy()) == pps.OK
    assert s.stats()["fallback_iteration"] >= 4
    assert s.get_error_compute_operator() <= 1e-10
    net.close()


def test_set_learned_rejects_unsupported(gpu):
    net = pps.UNet((16, 32, 64), seed=5)
    with pytest.raises(pps.PpsError):
        pps.FlexibleCG(pps.BlockGrid.cube(30), form="fp64").set_learned(net, 0, 1.0, FLAGS)   # 30 % 4 != 0
    with pytest.raises(pps.PpsError):
        pps.BiCGSTAB(pps.BlockGrid.cube(32), form="parity").set_learned(net, 0, 1.0, FLAGS)
    net.close()


def _restrict_1d(nf):
    """Full weighting along one axis: coarse c on fine 2c+1, weights 1/4, 1/2, 1/4."""
    r = np.zeros((nf // 2, nf))
    for c in range(nf // 2):
        for a, w in enumerate((0.25, 0.5, 0.25)):
            if 2 * c + a < nf:
                r[c, 2 * c + a] = w
    return r


def _along_axes(mats, f):
    return np.einsum("ai,bj,ck,ijk->abc", mats[0], mats[1], mats[2], f, optimize=True)


@pytest.mark.parametrize("form,m", [("fp64", 64), ("fp64", 128), ("mixed", 64)])
def test_learned_cycle_matches_its_composition(gpu, form, m):
    """apply_preconditioner with the network attached is the two-grid cycle
    z = Cheb(r); z += gain P^k N(R^k (r - A z)); z += Cheb(r - A z), rebuilt here from
    the plain Chebyshev application, the operator, numpy transfers and the network."""
    net = pps.UNet((16, 32, 64), seed=3, linear=True)
    k = int(round(math.log2(m / 32)))
    gain = 0.7
    grid = pps.BlockGrid.cube(m)
    b = learned.rhs(m, 30020, "field")
    plain = pps.FlexibleCG(grid, pps.ChebyshevIteration(11), form=form)
    s = pps.FlexibleCG(grid, pps.ChebyshevIteration(11), form=form)
    s.set_learned(net, k, gain, pps.LEARNED_PRECONDITIONER | pps.LEARNED_POST_SMOOTH)
    got = s.apply_preconditioner(b.copy())

    inner = (slice(2, m + 2),) * 3
    z = plain.apply_preconditioner(b.copy())
    res = np.zeros_like(b)
    res[inner] = (b - plain.apply_operator(z))[inner]
    coarse = res[inner]
    for _ in range(k):
        n = coarse.shape[0]
        coarse = _along_axes([_restrict_1d(n)] * 3, coarse)
    cin = torch.from_numpy(np.ascontiguousarray(coarse, np.float32)).cuda()
    cout = torch.empty_like(cin)
    net.forward(coarse.shape, cin.data_ptr(), cout.data_ptr(), normalize=True)
    corr = gain * cout.cpu().numpy().astype(np.float64)
    for _ in range(k):
        n = corr.shape[0]
        corr = _along_axes([2.0 * _restrict_1d(2 * n).T] * 3, corr)
    z[inner] += corr
    res2 = np.zeros_like(b)
    res2[inner] = (b - plain.apply_operator(z))[inner]
    z = z + plain.apply_preconditioner(res2)
    tol = 1e-4 if form == "fp64" else 2e-3
    assert rel_l2(got[inner], z[inner]) < tol
    s.close()
    plain.close()
    net.close()


def _lap(u, h):
    """The 7-point operator (u- - 2u + u+)/h^2 per axis, zero beyond the array."""
    p = np.pad(u, 1)
    out = -6.0 * u
    for ax in range(3):
        sl_m = [slice(1, -1)] * 3
        sl_p = [slice(1, -1)] * 3
        sl_m[ax] = slice(0, -2)
        sl_p[ax] = slice(2, None)
        out = out + p[tuple(sl_m)] + p[tuple(sl_p)]
    return out / (h * h)


def _cheb_smoother(b, h, ratio, n):
    """-s_{n-2} of the preconditioner's Chebyshev recurrence on [lmax/ratio, lmax]."""
    lmax = 12.0 / (h * h)
    lo = lmax / ratio
    theta, delta = (lo + lmax) / 2, (lo - lmax) / 2
    sigma = theta / delta
    if n == 2:
        return -b / theta
    rho_old = 1 / sigma
    rho = 1 / (2 * sigma - rho_old)
    s_prev = b / theta
    s = (2 * rho / delta) * (2 * b + _lap(b, h) / theta)
    for _ in range(2, n - 1):
        rho_old, rho = rho, 1 / (2 * sigma - rho)
        s, s_prev = rho * (2 * sigma * s + (2 / delta) * (b + _lap(s, h))) - rho * rho_old * s_prev, s
    return -s


def _level_lap(u, H, h):
    """The coarse-level operator: spacing H, lower wall H below the first unknown,
    upper wall h above the last (weights 2/(H(H+h)) and -2/(Hh) there)."""
    out = _lap(u, H)
    for ax in range(3):
        last = [slice(None)] * 3
        prev = [slice(None)] * 3
        last[ax] = -1
        prev[ax] = -2
        out[tuple(last)] += (2.0 / (H * (H + h)) - 1.0 / (H * H)) * u[tuple(prev)] \
            + (-2.0 / (H * h) + 2.0 / (H * H)) * u[tuple(last)]
    return out


def _level_diag(shape, H, h):
    d = np.zeros(shape)
    for ax in range(3):
        c = np.full(shape[ax], 2.0 / (H * H))
        c[-1] = 2.0 / (H * h)
        sh = [1, 1, 1]
        sh[ax] = shape[ax]
        d = d + c.reshape(sh)
    return d


def _jacobi_cheb(b, H, h, ratio, n):
    """-s_{n-2} of the Chebyshev recurrence on D^-1 A (D = -diag A) over [2/ratio, 2]."""
    dinv = 1.0 / _level_diag(b.shape, H, h)
    lo, hi = 2.0 / ratio, 2.0
    theta, delta = (lo + hi) / 2, (lo - hi) / 2
    sigma = theta / delta
    bb = dinv * b
    if n == 2:
        return -bb / theta
    rho_old = 1 / sigma
    rho = 1 / (2 * sigma - rho_old)
    s_prev = bb / theta
    s = rho * (2 * sigma * s_prev + (2 / delta) * dinv * (b + _level_lap(s_prev, H, h)))
    for _ in range(2, n - 1):
        rho_old, rho = rho, 1 / (2 * sigma - rho)
        s, s_prev = rho * (2 * sigma * s + (2 / delta) * dinv * (b + _level_lap(s, H, h))) - rho * rho_old * s_prev, s
    return -s


@pytest.mark.parametrize("form,m,fd,cd,coarse", [("fp64", 128, 3, 4, "network"), ("fp64", 64, 4, 0, "network"),
                                                  ("mixed", 128, 3, 4, "network"), ("fp64", 128, 3, 4, "exact"),
                                                  ("mixed", 128, 3, 4, "exact"), ("fp64", 128, 3, 4, "zero"),
                                                  ("fp64", 128, 3, 4, "smooth")])
def test_learned_vcycle_matches_its_composition(gpu, form, m, fd, cd, coarse):
    """The multigrid form of the learned cycle, rebuilt level by level in numpy:
    Chebyshev smoothing on [lmax/ratio, lmax] of the solver's grid, Jacobi-scaled
    Chebyshev on the coarse levels (spacing 2^l h, upper wall h above the last
    unknown), residual restriction, the coarsest level's solver (the network, or the
    alternatives of pps_set_coarse_solver: the exact level inverse, no correction,
    the coarse smoother), prolongation, post-smoothing."""
    net = pps.UNet((16, 32, 64), seed=4, linear=True)
    k = int(round(math.log2(m / 32)))
    gain, ratio = 0.6, 8.0
    grid = pps.BlockGrid.cube(m)
    b = learned.rhs(m, 30021, "blobs")
    s = pps.FlexibleCG(grid, pps.ChebyshevIteration(11), form=form)
    s.set_learned(net, k, gain, pps.LEARNED_PRECONDITIONER | pps.LEARNED_POST_SMOOTH)
    s.set_learned_cycle(fd, cd, ratio)
    kinds = {"network": pps.COARSE_NETWORK, "exact": pps.COARSE_EXACT, "zero": pps.COARSE_ZERO,
             "smooth": pps.COARSE_SMOOTH}
    s.set_coarse_solver(kinds[coarse])
    got = s.apply_preconditioner(b.copy())

    inner = (slice(2, m + 2),) * 3
    h = 1.0 / (m + 1)
    r0 = b[inner].copy()

    def restrict(f):
        return _along_axes([_restrict_1d(f.shape[0])] * 3, f)

    def prolong(c):
        return _along_axes([2.0 * _restrict_1d(2 * c.shape[0]).T] * 3, c)

    def network(r):
        if coarse == "exact":   # A_k^-1 r: spacing 2^k h, upper wall h above the last unknown
            return learned.level_solve(torch.from_numpy(r), h * 2 ** k, 2.0 ** -k).numpy()
        if coarse == "zero":
            return np.zeros_like(r)
        if coarse == "smooth":
            return _jacobi_cheb(r, h * 2 ** k, h, ratio, cd)
        cin = torch.from_numpy(np.ascontiguousarray(r, np.float32)).cuda()
        cout = torch.empty_like(cin)
        net.forward(r.shape, cin.data_ptr(), cout.data_ptr(), normalize=True)
        return gain * cout.cpu().numpy().astype(np.float64)

    X = _cheb_smoother(r0, h, ratio, fd)
    r = restrict(r0 - _lap(X, h))
    rs, zs = [None], [None]
    for lvl in range(1, k):
        hl = h * 2 ** lvl
        z = _jacobi_cheb(r, hl, h, ratio, cd) if cd else np.zeros_like(r)
        rs.append(r)
        zs.append(z)
        r = restrict(r - _level_lap(z, hl, h)) if cd else restrict(r)
    e = network(r)
    for lvl in range(k - 1, 0, -1):
        hl = h * 2 ** lvl
        z = zs[lvl] + prolong(e)
        if cd:
            z = z + _jacobi_cheb(rs[lvl] - _level_lap(z, hl, h), hl, h, ratio, cd)
        e = z
    X = X + prolong(e)
    X = X + _cheb_smoother(r0 - _lap(X, h), h, ratio, fd)
    tol = 1e-4 if form == "fp64" else 2e-3
    assert rel_l2(got[inner], X) < tol
    s.close()
    net.close()


def test_learned_vcycle_solve_with_and_without_fused_dots(gpu):
    """Flexible CG with the learned V-cycle.  On the x-vectorised FP32 tiles the
    cycle's last prolongation also sums z.r and z.Ap; on one- and two-column tiles a
    separate kernel sums them (the prolongation itself then runs on one-column tiles
    of the whole grid).  All solves meet the FP64 tolerance without falling back, with
    the same iteration count (+-1), and agree to well below the tolerance's reach."""
    m = 64
    k = int(round(math.log2(m / 16)))
    train = learned.make_dataset(16, range(10000, 10032), coarsen=k)
    scale = learned.fit_scale(train)
    net = pps.UNet((16, 32, 64), seed=1, linear=True)
    learned.train(net, train, scale, 300, lr=1e-3)
    gain = scale * ((2 ** k / (m + 1)) / (1.0 / 17)) ** 2
    b = learned.rhs(m, 30011, "field")
    out = []
    for cx in (4, 1, 2):
        s = pps.FlexibleCG(pps.BlockGrid.cube(m), pps.ChebyshevIteration(11), tolerance=1e-10, form="mixed",
                           inner_tol=1e-5)
        s.set_learned(net, k, gain, pps.LEARNED_PRECONDITIONER)
        s.set_learned_cycle(5, 4, 8.0)
        s.set_tuning({**s.tuning(), "cheb_cx": cx})
        x = np.zeros_like(b)
        assert s(x, b.copy()) == pps.OK
        st = s.stats()
        assert st["fallback_iteration"] == -1 and st["learned_applications"] > 0
        assert s.get_error_compute_operator() <= 1e-10
        out.append((x, s.get_num_iteration_final()))
        s.close()
    net.close()
    for x, it in out[1:]:
        assert abs(out[0][1] - it) <= 1, (out[0][1], it)
        assert rel_l2(out[0][0], x) < 1e-7
