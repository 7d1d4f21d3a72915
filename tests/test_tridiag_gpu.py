"""GPU parity of the batched tridiagonal integrator and the diffusion stage,
called through the C ABI (libember_gpu.so), against the CPU oracle and the
reference's own golden table / property tests."""
import json
import os

import numpy as np
import pytest

import oracle
from ember_gb300 import _lib as L
from ember_gb300.diffusion import FlameGrid, TridiagonalIntegratorBatch, integrate_diffusion_terms

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def golden(golden_dir):
    with open(os.path.join(golden_dir, "tridiag_bdf.json")) as f:
        return json.load(f)


def _golden_batch(g, copies=3):
    b = TridiagonalIntegratorBatch([5] * copies)
    rep = lambda v: np.tile(np.asarray(v, dtype=float), copies)
    b.set_coefficients(rep(g["a"]), rep(g["b"]), rep(g["c"]), rep(g["k"]))
    b.set_y0(rep(g["y0"]))
    return b


def test_golden_stepwise(gpu_lib, golden):
    b = _golden_batch(golden)
    b.initialize(0.0, 0.2)
    for j, row in enumerate(golden["table_cpp"]):
        for y in b.split(b.y):
            np.testing.assert_allclose(y, row, rtol=0, atol=1e-10)
        b.step()


def test_golden_full_and_short(gpu_lib, golden):
    b = _golden_batch(golden)
    b.initialize(0.0, 0.2)
    b.integrate_to_time(1.0)
    y, t, h = b.state()
    np.testing.assert_allclose(t, 1.0, atol=1e-10)
    np.testing.assert_allclose(h, 0.2, atol=1e-10)
    for ys in b.split(y):
        np.testing.assert_allclose(ys, golden["table_cpp"][5], rtol=0, atol=1e-10)
    b.set_y0(np.tile(golden["y0"], 3))
    b.initialize(0.0, 1.3)
    b.integrate_to_time(0.2)
    y, t, h = b.state()
    np.testing.assert_allclose(t, 0.2, atol=1e-10)
    for ys in b.split(y):
        np.testing.assert_allclose(ys, golden["table_cpp"][1], rtol=0, atol=1e-10)


def _random_systems(rng, n_sys, nmax):
    sizes = rng.integers(2, nmax, n_sys)
    sys = []
    for n in sizes:
        a = rng.uniform(0.1, 1.0, n)
        c = rng.uniform(0.1, 1.0, n)
        b = -(a + c) * rng.uniform(1.0, 1.5, n)
        k = rng.normal(size=n)
        y0 = rng.normal(size=n)
        sys.append((a, b, c, k, y0))
    return sizes, sys


def test_batch_bitwise_vs_oracle(gpu_lib):
    rng = np.random.default_rng(11)
    sizes, sys = _random_systems(rng, 40, 300)
    b = TridiagonalIntegratorBatch(sizes)
    cat = lambda i: np.concatenate([s[i] for s in sys])
    b.set_coefficients(cat(0), cat(1), cat(2), cat(3))
    b.set_y0(cat(4))
    h0 = rng.uniform(0.01, 0.3, len(sizes))
    t_end = rng.uniform(0.05, 2.0, len(sizes))
    b.initialize(0.0, h0)
    b.integrate_to_time(t_end)
    y, t, h = b.state()
    for i, (ys, s) in enumerate(zip(b.split(y), sys)):
        yo, to, ho = oracle.tridiag_run(*s, 0.0, h0[i], t_end=t_end[i])
        assert np.array_equal(ys, yo), f"system {i} differs"
        assert t[i] == to and h[i] == ho
    # ydot of the final state
    ydot = b.get_ydot()
    for ys_dot, ys, s in zip(b.split(ydot), b.split(y), sys):
        a, bb, c, k = s[:4]
        ref = bb * ys + k
        ref[1:] += a[1:] * ys[:-1]
        ref[:-1] += c[:-1] * ys[1:]
        np.testing.assert_allclose(ys_dot, ref, rtol=1e-12, atol=1e-12)


def test_stepwise_matches_integrate(gpu_lib):
    rng = np.random.default_rng(5)
    sizes, sys = _random_systems(rng, 8, 50)
    b = TridiagonalIntegratorBatch(sizes)
    cat = lambda i: np.concatenate([s[i] for s in sys])
    b.set_coefficients(cat(0), cat(1), cat(2), cat(3))
    b.set_y0(cat(4))
    b.initialize(0.0, 0.1)
    for _ in range(4):
        b.step()
    y, t, h = b.state()
    for i, (ys, s) in enumerate(zip(b.split(y), sys)):
        yo, to, _ = oracle.tridiag_run(*s, 0.0, 0.1, n_steps=4)
        assert np.array_equal(ys, yo)


# ---- diffusion stage -------------------------------------------------------

def _flame(rng, n, left, right, alpha, spread=0.4, max_ratio=None):
    walk = np.cumsum(rng.uniform(-spread, spread, n - 1))
    if max_ratio is not None:  # keep the smallest spacing (and the step-size rule's h) bounded
        walk = np.clip(walk, -np.log(max_ratio), np.log(max_ratio))
    dx = rng.uniform(1e-5, 1e-4) * np.exp(walk)
    x = np.concatenate([[rng.uniform(0.0, 1e-3) if alpha else -1e-3], dx]).cumsum()
    return FlameGrid(x=x, left_bc=left, right_bc=right, alpha=alpha)


def _diffusion_case(rng, n_flames, n_vars, nmin, nmax, all_bcs=True, **grid_kw):
    grids = []
    for f in range(n_flames):
        n = int(rng.integers(nmin, nmax + 1))
        left = int(rng.integers(0, 5)) if all_bcs else 0
        right = int(rng.choice([0, 1, 4])) if all_bcs else 0
        grids.append(_flame(rng, n, left, right, int(rng.integers(0, 2)) if all_bcs else 0, **grid_kw))
    B = [np.exp(rng.uniform(-1, 1, (n_vars, g.n_points))) for g in grids]
    D = [np.exp(rng.uniform(np.log(1e-6), np.log(1e-3), (n_vars, g.n_points))) for g in grids]
    S = [rng.normal(scale=10.0, size=(n_vars, g.n_points)) for g in grids]
    Y = [np.cumsum(rng.normal(size=(n_vars, g.n_points)), axis=1) for g in grids]
    return grids, B, D, S, Y


def _oracle_stage(grids, B, D, S, Y, t0, t1, h=None, wall=None, yinf=None, mult=10.0, gdt=2e-5):
    out = []
    n_vars = Y[0].shape[0]
    for f, g in enumerate(grids):
        yf = np.empty_like(Y[f])
        for v in range(n_vars):
            i = f * n_vars + v
            yf[v] = oracle.diffusion_system(g.x, B[f][v], D[f][v], Y[f][v], t0, t1, split_const=S[f][v],
                                            alpha=g.alpha, left_bc=g.left_bc, right_bc=g.right_bc,
                                            wall_const=0.0 if wall is None else wall[i],
                                            y_inf=0.0 if yinf is None else yinf[i],
                                            h=0.0 if h is None else h[i], mult=mult, gdt=gdt)
        out.append(yf)
    return out


@pytest.mark.parametrize("explicit_h", [False, True])
def test_diffusion_stage_bitwise_vs_oracle(gpu_lib, explicit_h):
    rng = np.random.default_rng(2024 + explicit_h)
    n_flames, n_vars = 12, 7
    grids, B, D, S, Y = _diffusion_case(rng, n_flames, n_vars, 3, 120)
    nsys = n_flames * n_vars
    h = rng.uniform(1e-7, 4e-6, nsys) if explicit_h else None
    wall = rng.uniform(0, 5, nsys)
    yinf = rng.normal(size=nsys)
    t0, t1 = 1e-3, 1e-3 + 1e-5
    out, status = integrate_diffusion_terms(grids, B, D, S, Y, t0, t1, h=h, wall_const=wall, y_inf=yinf,
                                            algorithm=L.DIFFUSION_SERIAL)
    assert (np.asarray(status) == 0).all()
    ref = _oracle_stage(grids, B, D, S, Y, t0, t1, h=h, wall=wall, yinf=yinf)
    for f in range(n_flames):
        assert np.array_equal(out[f], ref[f]), f"flame {f} (bc {grids[f].left_bc},{grids[f].right_bc}) differs"


# The warp-parallel solver re-associates the Thomas algorithm (chunk carries
# by prefix scans, 1/den folded into the coefficients), so it agrees with the
# reference to rounding, not bit for bit. The reference's own rounding error
# on these systems, measured against the same recurrences in 80-bit extended
# precision, reaches 1.6e-13 of max|y| (many BDF2 steps of a stiff,
# ControlVolume-bounded system), so the bound per system is
# |y_gpu - y_ref| <= 1e-12 * max|y_ref|.
PARALLEL_TOL = 1e-12


def _assert_close_per_system(out, ref, what):
    for v in range(ref.shape[0]):
        scale = np.abs(ref[v]).max()
        err = np.abs(out[v] - ref[v]).max()
        assert err <= PARALLEL_TOL * scale, f"{what}, variable {v}: max error {err:.3e} vs max|y| {scale:.3e}"


@pytest.mark.parametrize("explicit_h", [False, True])
def test_diffusion_stage_parallel_vs_oracle(gpu_lib, explicit_h):
    rng = np.random.default_rng(4048 + explicit_h)
    n_flames, n_vars = 14, 5
    grids, B, D, S, Y = _diffusion_case(rng, n_flames, n_vars, 3, 700, spread=0.1, max_ratio=4.0)
    nsys = n_flames * n_vars
    h = rng.uniform(1e-7, 4e-6, nsys) if explicit_h else None  # 3 to 100 steps: BDF1 x 8, then BDF2
    wall = rng.uniform(0, 5, nsys)
    yinf = rng.normal(size=nsys)
    t0, t1 = 1e-3, 1e-3 + 1e-5
    out, status = integrate_diffusion_terms(grids, B, D, S, Y, t0, t1, h=h, wall_const=wall, y_inf=yinf)
    assert (np.asarray(status) == 0).all()
    ref = _oracle_stage(grids, B, D, S, Y, t0, t1, h=h, wall=wall, yinf=yinf)
    for f in range(n_flames):
        _assert_close_per_system(out[f], ref[f], f"flame {f} (N {grids[f].n_points}, bc {grids[f].left_bc},"
                                                 f"{grids[f].right_bc}, alpha {grids[f].alpha})")


def test_diffusion_parallel_long_grid(gpu_lib):
    # 20000 points: 625 points per lane, many Moebius renormalisations.
    rng = np.random.default_rng(31)
    grids, B, D, S, Y = _diffusion_case(rng, 1, 3, 20000, 20000, spread=0.1, max_ratio=4.0)
    out, status = integrate_diffusion_terms(grids, B, D, S, Y, 0.0, 1e-5, h=[1e-5, 2e-6, 1e-5])
    assert (np.asarray(status) == 0).all()
    ref = _oracle_stage(grids, B, D, S, Y, 0.0, 1e-5, h=[1e-5, 2e-6, 1e-5])
    _assert_close_per_system(out[0], ref[0], "20000-point flame")


def test_diffusion_reference_properties_on_gpu(gpu_lib):
    # test/test_diffusionSystem.cpp Gaussian and Superposition2, through the GPU stage.
    n = 401
    x = np.linspace(-2, 2, n)
    g = FlameGrid(x=x)
    t0, t = 0.2, 0.3
    y0 = np.exp(-x * x / (4 * 0.1 * t0))
    out, st = integrate_diffusion_terms([g], [np.ones((1, n))], [np.full((1, n), 0.1)], [np.zeros((1, n))],
                                        [y0[None, :]], t0, t, h=[0.001])
    exact = np.sqrt(t0 / t) * np.exp(-x * x / (4 * 0.1 * t))
    np.testing.assert_allclose(out[0][0], exact, atol=1e-4)
    Dv, Bv = 0.1 + 0.02 * x, 1 + 0.5 * x * x
    ya, yb = np.cos(np.pi * x), np.sin(np.pi * x / 4.0)
    Y = [np.stack([ya, yb, ya + yb])]
    out, st = integrate_diffusion_terms([g], [np.tile(Bv, (3, 1))], [np.tile(Dv, (3, 1))], [np.zeros((3, n))],
                                        Y, 0.0, 0.1, h=[0.001] * 3)
    np.testing.assert_allclose(out[0][0] + out[0][1], out[0][2], atol=1e-12)


def test_diffusion_device_memory_matches_host(gpu_lib):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(9)
    grids, B, D, S, Y = _diffusion_case(rng, 5, 4, 50, 300)
    host, _ = integrate_diffusion_terms(grids, B, D, S, [y.copy() for y in Y], 0.0, 1e-5)
    flat = lambda arrs: torch.as_tensor(np.concatenate([a.reshape(-1) for a in arrs]), device="cuda")
    yd = flat(Y)
    integrate_diffusion_terms(grids, flat(B), flat(D), flat(S), yd, 0.0, 1e-5)
    torch.cuda.synchronize()
    assert np.array_equal(yd.cpu().numpy(), np.concatenate([h.reshape(-1) for h in host]))


def test_diffusion_large_flames_c3_subset(gpu_lib):
    # Config-3 shapes: 55 variables, grids of 3000-4000 points whose spacing
    # varies by at most 16x, dt = 1e-5.
    rng = np.random.default_rng(77)
    grids, B, D, S, Y = _diffusion_case(rng, 3, 55, 3000, 4000, all_bcs=False, spread=0.1, max_ratio=4.0)
    S = [np.zeros_like(s) for s in S]
    h = np.full(3 * 55, 1e-5)
    out, status = integrate_diffusion_terms(grids, B, D, S, Y, 0.0, 1e-5, h=h)
    assert (np.asarray(status) == 0).all()
    for f in range(3):
        for v in (0, 17, 54):
            ref = oracle.diffusion_system(grids[f].x, B[f][v], D[f][v], Y[f][v], 0.0, 1e-5, h=1e-5)
            _assert_close_per_system(out[f][v][None, :], ref[None, :], f"flame {f}")


@pytest.mark.parametrize("algorithm", [L.DIFFUSION_PARALLEL, L.DIFFUSION_SERIAL])
def test_diffusion_extreme_grid_vs_extended_precision(gpu_lib, algorithm):
    # Grids whose spacing spans 1e-13 to 1e-1 m: matrix coefficients reach
    # 1e23 against a BDF shift of 8e5, so b - shift keeps none of the shift and
    # the reference's own result is off by up to 1e-10 of max|y|. The
    # parallel solver carries the pivots in u = 1 + lu_c with positive terms
    # only and stays within 1e-12 of the exact solution of the same discrete
    # problem (extended-precision restatement); the serial one reproduces the
    # reference bit for bit, so it is held to the reference's own error.
    from oracle import extended
    rng = np.random.default_rng(77)
    grids, B, D, S, Y = _diffusion_case(rng, 3, 55, 3000, 4000, all_bcs=False)
    S = [np.zeros_like(s) for s in S]
    out, status = integrate_diffusion_terms(grids, B, D, S, Y, 0.0, 1e-5, h=np.full(3 * 55, 1e-5),
                                            algorithm=algorithm)
    assert (np.asarray(status) == 0).all()
    worst_ref = 0.0
    for f in range(3):
        for v in (0, 54):
            exact = extended.diffusion_system(grids[f].x, B[f][v], D[f][v], Y[f][v], 0.0, 1e-5, 1e-5)
            ref = oracle.diffusion_system(grids[f].x, B[f][v], D[f][v], Y[f][v], 0.0, 1e-5, h=1e-5)
            scale = np.abs(exact).max()
            err_ref = np.abs(ref - exact).max() / scale
            err = np.abs(out[f][v] - exact).max() / scale
            worst_ref = max(worst_ref, err_ref)
            if algorithm == L.DIFFUSION_PARALLEL:
                assert err <= 1e-12, f"flame {f} var {v}: {err:.3e} of max|y| from the exact solution"
            else:
                assert np.array_equal(out[f][v], ref)
    assert worst_ref > 1e-11  # the case does exercise the reference's rounding limit


def test_bad_step_reports_status(gpu_lib):
    rng = np.random.default_rng(1)
    grids, B, D, S, Y = _diffusion_case(rng, 2, 2, 10, 20)
    h = np.array([1e-6, -1.0, 1e-6, 1e-6])
    out, status = integrate_diffusion_terms(grids, B, D, S, Y, 0.0, 1e-5, h=h)
    assert list(np.asarray(status)) == [0, -1, 0, 0]


@pytest.mark.parametrize("algorithm", [L.DIFFUSION_PARALLEL, L.DIFFUSION_SERIAL])
def test_diffusion_minimal_grids(gpu_lib, algorithm):
    # Three-point grids (the smallest the stage accepts) with every boundary
    # pair, and 31/32/33-point grids around one point per lane.
    rng = np.random.default_rng(12)
    grids = []
    for left in range(5):
        for right in (0, 1, 4):
            grids.append(_flame(rng, 3, left, right, left % 2))
    for n in (31, 32, 33):
        grids.append(_flame(rng, n, 0, 0, 0))
    n_vars = 2
    B = [np.exp(rng.uniform(-1, 1, (n_vars, g.n_points))) for g in grids]
    D = [np.exp(rng.uniform(np.log(1e-6), np.log(1e-4), (n_vars, g.n_points))) for g in grids]
    S = [rng.normal(size=(n_vars, g.n_points)) for g in grids]
    Y = [rng.normal(size=(n_vars, g.n_points)) for g in grids]
    h = np.full(len(grids) * n_vars, 2e-6)
    out, status = integrate_diffusion_terms(grids, B, D, S, Y, 0.0, 1e-5, h=h, algorithm=algorithm)
    assert (np.asarray(status) == 0).all()
    ref = _oracle_stage(grids, B, D, S, Y, 0.0, 1e-5, h=h)
    for f in range(len(grids)):
        if algorithm == L.DIFFUSION_SERIAL:
            assert np.array_equal(out[f], ref[f])
        else:
            _assert_close_per_system(out[f], ref[f], f"grid {f}")


@pytest.mark.parametrize("algorithm", [L.DIFFUSION_PARALLEL, L.DIFFUSION_SERIAL])
def test_diffusion_pinned_host_call_matches_device_call(gpu_lib, algorithm):
    # A large host-memory call on page-locked arrays runs as groups of flames
    # whose copies overlap each other's kernels; every system must come out as
    # from the single-group call on device arrays (and from pageable arrays),
    # statuses included, with explicit h, wall constants and y_inf per system.
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(21)
    n_vars = 20
    grids, B, D, S, Y = _diffusion_case(rng, 16, n_vars, 2800, 4000, spread=0.1, max_ratio=4.0)
    n_sys = 16 * n_vars
    h = np.full(n_sys, 2.5e-6)
    wall = rng.uniform(0.0, 1e3, n_sys)
    yinf = rng.normal(size=n_sys)
    flat = lambda arrs: np.concatenate([a.reshape(-1) for a in arrs])
    assert flat(Y).size >= 1 << 20
    dev = lambda a: torch.as_tensor(a, device="cuda")
    yd = dev(flat(Y))
    _, st_dev = integrate_diffusion_terms(grids, dev(flat(B)), dev(flat(D)), dev(flat(S)), yd, 0.0, 1e-5,
                                          h=dev(h), wall_const=dev(wall), y_inf=dev(yinf), algorithm=algorithm)
    torch.cuda.synchronize()
    ref = yd.cpu().numpy()
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    yp = pin(flat(Y))
    _, st_pin = integrate_diffusion_terms(grids, pin(flat(B)), pin(flat(D)), pin(flat(S)), yp, 0.0, 1e-5, h=h,
                                          wall_const=wall, y_inf=yinf, algorithm=algorithm)
    yq = flat(Y).copy()
    _, st_page = integrate_diffusion_terms(grids, flat(B), flat(D), flat(S), yq, 0.0, 1e-5, h=h, wall_const=wall,
                                           y_inf=yinf, algorithm=algorithm)
    assert np.isfinite(ref).all()
    assert np.array_equal(yp, ref) and np.array_equal(yq, ref)
    assert np.array_equal(np.asarray(st_pin), st_dev.cpu().numpy())
    assert np.array_equal(np.asarray(st_pin), np.asarray(st_page))
