"""Pins the C restatement (oracle/g4oracle.c) to the GENESIS 1.3 v4 reference.

The fixtures in tests/golden/ were produced by the reference itself, compiled from
its own sources (tests/golden/gen_golden.py). The oracle is bit-exact with them on
x86-64 (same C library, no fused multiply-add); elsewhere a 1e-14 relative bound
covers last-bit differences of the platform's log/exp/sin.
"""
import platform

import numpy as np
import pytest

from conftest import golden

EXACT = platform.machine() in ("x86_64", "AMD64")


def same(a, b, rtol=1e-14):
    if EXACT:
        return np.array_equal(a, b)
    return np.allclose(a, b, rtol=rtol, atol=0)


def test_ran2_and_hammersley_streams(oracle):
    d = golden("streams.npz")
    for s in (1, 7, 11, 123456789):
        assert np.array_equal(oracle.ran2(s, 64), d[f"ran2_{s}"]), s  # integer arithmetic: exact
    for b in range(6):
        for st in (0, 12345, 987654321):
            assert np.array_equal(oracle.hammersley(b, st, 64), d[f"ham_{b}_{st}"]), (b, st)


def test_inverfc_bessel_fc(oracle):
    d = golden("streams.npz")
    assert same(oracle.inverfc(d["inverfc_x"]), d["inverfc_y"])
    xs = d["bessel_x"]
    got = np.array([[oracle.besselj(n, v) for v in xs] for n in range(5)])
    assert same(got, d["bessel_j"])
    fc = np.array([[[oracle.fc(a, hel, h) for h in range(1, 8)] for hel in (0, 1)] for a in d["fc_aw"]])
    assert same(fc, d["fc"])
    # even harmonics of a planar undulator and harmonics > 1 of a helical one couple to 0
    assert np.all(d["fc"][:, 0, 1::2] == 0) and np.all(d["fc"][:, 1, 1:] == 0)


@pytest.mark.parametrize("name", ["quiet_nb4", "shot_nb4", "shot_nb8", "bunch_emod", "shot_profile"])
def test_quiet_loading_and_shot_noise(oracle, name):
    d = golden("loading.npz")
    islice0, npart, nbins, seed, sn = (int(v) for v in d[name + "_args"])
    got = oracle.load_beam(d[name + "_sp"], islice0, npart, nbins, seed, sn, 1e-10, 1.0)
    assert same(got, d[name])


@pytest.mark.parametrize("name", ["gh_fund", "gh_h3"])
def test_gauss_hermite(oracle, name):
    d = golden("loading.npz")
    gm, ng = d[name + "_grid"]
    assert same(oracle.gauss_hermite(d[name + "_par"], gm, int(ng)), d[name])


@pytest.mark.parametrize("case", ["planar", "helical", "harm13", "steady"])
@pytest.mark.parametrize("stages", [1, 2, 4, 7])
def test_integration_steps(oracle, case, stages):
    d = golden("steps.npz")
    g = lambda k: d[f"{case}_{k}"]
    gammaref, time_run, periodic = g("args")
    lat = g("lat")[:1] if stages != 7 else g("lat")
    part, fld, first, _ = oracle.run_steps(lat, gammaref, g("part"), g("cur"), 1e-10, 1.0, g("harm"),
                                           g("gridmax"), g("fields"), g("first"),
                                           time_run=int(time_run), periodic=int(periodic),
                                           stages=stages)
    assert same(part, g(f"s{stages}_part"), rtol=1e-12)
    assert same(fld, g(f"s{stages}_fields"), rtol=1e-12)
    assert np.array_equal(first, g(f"s{stages}_first"))


def test_threads_do_not_change_results(oracle):
    d = golden("steps.npz")
    g = lambda k: d[f"harm13_{k}"]
    args = (g("lat"), 11357.8, g("part"), g("cur"), 1e-10, 1.0, g("harm"), g("gridmax"), g("fields"), g("first"))
    a = oracle.run_steps(*args, periodic=1, nthreads=1)
    b = oracle.run_steps(*args, periodic=1, nthreads=3)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def _gauss_field(oracle, d):
    ng = int(d["ngrid"])
    par = np.array([d["lambda0"], d["power0"], 0, 0, d["waist"], 0, 0, 0, 0, 0, 0, 1.0])
    return oracle.gauss_hermite(par, float(d["gridmax"]), ng)


def test_config0_deck_final_power(oracle):
    """The 443-step planar FODO deck, steady state (the reference's genesis4 output)."""
    d = golden("config0.npz")
    fld = _gauss_field(oracle, d)[None, None]
    part, f, first, _ = oracle.run_steps(d["lat"], float(d["gammaref"]), d["beam"], d["current"], 1e-10,
                                         1.0, [1], [float(d["gridmax"])], fld, [0], time_run=0)
    df = oracle.diag_field(f[0], float(d["gridmax"]), 1e-10, 1, 0)
    db = oracle.diag_beam(part, 1)
    assert same(df[0, 0], d["power"][-1], rtol=1e-12)
    assert same(db[0, 24], d["bunching"][-1], rtol=1e-9)


def test_example1_deck_final_power(oracle):
    """Example1 of the reference (helical, lasing): 1104 steps, ngrid 255."""
    d = golden("example1.npz")
    fld = _gauss_field(oracle, d)[None, None]
    part, f, first, _ = oracle.run_steps(d["lat"], float(d["gammaref"]), d["beam"], d["current"], 1e-10,
                                         1.0, [1], [float(d["gridmax"])], fld, [0], time_run=0)
    df = oracle.diag_field(f[0], float(d["gridmax"]), 1e-10, 1, 0)
    assert same(df[0, 0], d["power"][-1], rtol=1e-12)
    # the reference's CI golden value (examples/Example1-SteadyState/TEST_power.py:14,17)
    assert abs(df[0, 0] / 0.932785e9 - 1) < 0.3


def _k2_and_sigmoid(n, dgrid, xks, xc=1.0, yc=1.0, sig=1.0):
    """Im(K2) and the source filter on the FFT index, FieldSolverFFT.cpp:131-145."""
    dk = 4.0 * np.arcsin(1.0) / (n * dgrid)
    shift = -0.5 * (n - 1)
    k2 = np.zeros((n, n))
    sg = np.zeros((n, n))
    for iy in range(n):
        dy = iy + shift
        y = dy / n / yc
        for ix in range(n):
            dx = ix + shift
            x = dx / n / xc
            iiy, iix = (iy + (n + 1) // 2) % n, (ix + (n + 1) // 2) % n
            k2[iiy, iix] = -(dx * dx + dy * dy) * dk * dk / 2.0 / xks
            sg[iiy, iix] = 1.0 / (1.0 + np.exp((np.sqrt(x * x + y * y) - 1) / sig))
    return k2, sg


@pytest.mark.parametrize("n", [15, 16, 21])
def test_fft_solver_matches_numpy(oracle, n):
    """The FFT solver of the oracle against numpy's pocketfft, a second transform
    besides the reference's (test_fft_solver_matches_reference): u' = IFFT(FFT(u)
    exp(K2 dz)) + 2 src, and the filtered form IFFT(FFT(u) exp(K2 dz) + 2 FFT(src)
    sigmoid)."""
    import g4cases as T
    rng = np.random.default_rng(n)
    ns, gm, dz = 2, 5e-5, 0.015
    u = (rng.standard_normal((1, ns, n * n)) + 1j * rng.standard_normal((1, ns, n * n))) * 1e3
    dgrid = 2 * gm / (n - 1)
    xks = 4.0 * np.arcsin(1.0) / 1e-10
    k2, sg = _k2_and_sigmoid(n, dgrid, xks, 0.7, 0.9, 0.3)
    prop = np.exp(1j * k2 * dz)
    # a drift step: no source
    lat = T.undulator_lattice(1.7, 0.015, 1, 1, 1e-10, 11357.8)
    lat[0, T.C["aw"]] = 0.0
    part = oracle.load_beam(T.slice_params(ns, 11357.8, 2.0, 0.4e-6, 15.0), 0, 32, 4, 1, 0, 1e-10, 1.0)
    cur = np.full(ns, 3000.0)
    _, f1, _, _ = oracle.run_steps(lat, 11357.8, part, cur, 1e-10, 1.0, [1], [gm], u, [0], stages=2, solver=1)
    for s in range(ns):
        want = np.fft.ifft2(np.fft.fft2(u[0, s].reshape(n, n)) * prop).ravel()
        assert np.allclose(f1[0, s], want, rtol=0, atol=1e-12 * np.abs(want).max())
    # an undulator step: source deposited; the filtered solve against numpy
    lat[0, T.C["aw"]] = 1.7
    _, fu, _, _ = oracle.run_steps(lat, 11357.8, part, cur, 1e-10, 1.0, [1], [gm], u, [0], stages=2, solver=1)
    _, ff, _, _ = oracle.run_steps(lat, 11357.8, part, cur, 1e-10, 1.0, [1], [gm], u, [0], stages=2, solver=2,
                                   filt=[0.7, 0.9, 0.3])
    for s in range(ns):
        free = np.fft.ifft2(np.fft.fft2(u[0, s].reshape(n, n)) * prop)
        src = (fu[0, s].reshape(n, n) - free) / 2
        assert np.abs(src).max() > 0
        want = np.fft.ifft2(np.fft.fft2(u[0, s].reshape(n, n)) * prop + 2 * np.fft.fft2(src) * sg).ravel()
        assert np.allclose(ff[0, s], want, rtol=0, atol=1e-10 * np.abs(want).max())


@pytest.mark.parametrize("n", [15, 16, 21])
def test_far_field_moments_match_numpy(oracle, n):
    """The oracle's far-field pointing and divergence (DiagField with FFTW,
    Diagnostic.cpp:786-847) against numpy, besides the reference: the power-weighted
    moments of |FFT2(u)|^2 on the shifted frequency map, scaled by
    xlambda / (ngrid dgrid), by window slice."""
    rng = np.random.default_rng(n + 100)
    ns, gm, lam, harm, first = 3, 5e-5, 1e-10, 3, 1
    x = np.arange(n) - 0.5 * (n - 1)
    g = np.exp(-((x[None, :] - 1.3) ** 2 + (x[:, None] + 0.7) ** 2) / (0.2 * n * n))
    u = np.stack([(g * np.exp(1j * (0.3 * s + 0.2) * x[None, :])
                   + 0.01 * (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))).ravel()
                  for s in range(ns)])
    got = oracle.diag_field_fft(u, gm, lam, harm, first)
    dgrid = 2 * gm / (n - 1)
    sclt = lam / harm / n / dgrid
    for is0 in range(ns):
        F = np.fft.fft2(u[is0].reshape(n, n))
        idx = (np.arange(n) + (n + 1) // 2) % n
        w = np.abs(F[np.ix_(idx, idx)]) ** 2  # [iy, ix] on the shifted map
        p = w.sum()
        fx1, fx2 = (w * x[None, :]).sum() / p, (w * x[None, :] ** 2).sum() / p
        fy1, fy2 = (w * x[:, None]).sum() / p, (w * x[:, None] ** 2).sum() / p
        want = [fx1 * sclt, np.sqrt(abs(fx2 - fx1 * fx1)) * sclt, fy1 * sclt, np.sqrt(abs(fy2 - fy1 * fy1)) * sclt]
        is_ = (ns + is0 - first) % ns
        assert np.allclose(got[is_], want, rtol=1e-10, atol=1e-12 * max(abs(v) for v in want))


FFT_CASES = [f"n{n}_s{s}" for n in (25, 32, 45, 22, 38) for s in (1, 2)] + ["harm255"]


def fft_case_inputs(d, name, gauss_hermite):
    """Inputs of one case of tests/golden/fft.npz: (lattice, particles, current, harm,
    gridmax, fields, solver, filter); the ngrid-255 case's fields are rebuilt with the
    given Gauss-Hermite loader (bit-exact with the reference's, loading.npz)."""
    import gen_golden
    g = lambda k: d[f"{name}_{k}"]
    if name == "harm255":
        fld = gen_golden.harm255_fields(gauss_hermite)
    else:
        fld = d[f"{name.split('_')[0]}_fields"]
    return g("lat"), g("part"), g("cur"), g("harm"), g("gridmax"), fld, int(g("solver")), g("filt")


@pytest.mark.parametrize("case", FFT_CASES)
def test_fft_solver_matches_reference(oracle, case):
    """The oracle's FFT field solver against the reference's own FieldSolverFFT
    (FieldSolverFFT.cpp:9-167) built with -DFFTW on the FFTW stand-in of
    oracle/ref_build (tests/golden/fft.npz): whole lattices (13 and 11 steps) of
    periodic time-dependent windows, two or three harmonics, unfiltered and filtered
    sources, odd and even grids and ngrid 255. The two transforms round differently
    (FFTW's documented DFT evaluated exactly against the oracle's mixed-radix FFT):
    within 1e-13 of the largest field value, particles within 1e-13."""
    import gen_golden
    d = golden("fft.npz")
    lat, part, cur, harm, gm, fld, solver, filt = fft_case_inputs(d, case, oracle.gauss_hermite)
    p, f, first, _ = oracle.run_steps(lat, 11357.8, part, cur, 1e-10, 1.0, harm, gm, fld, [0] * len(harm),
                                      periodic=1, solver=solver, filt=filt, nthreads=8)
    want_f = d[f"{case}_out_fields"]
    if case == "harm255":
        f = f[:, :, gen_golden.HARM255_CELLS]
    assert np.array_equal(first, d[f"{case}_out_first"])
    for k in range(len(harm)):
        assert np.abs(want_f[k]).max() > 0
        assert np.abs(f[k] - want_f[k]).max() <= 1e-13 * np.abs(want_f[k]).max(), k
    want_p = d[f"{case}_out_part"]
    for col in range(6):
        assert np.abs(p[..., col] - want_p[..., col]).max() <= 1e-13 * np.abs(want_p[..., col]).max(), col


@pytest.mark.parametrize("ng,harm,first", [(45, 1, 0), (32, 3, 2), (51, 1, 5), (21, 5, 1)])
def test_far_field_matches_reference(oracle, ng, harm, first):
    """The oracle's field diagnostics against the reference's DiagField::getValues
    with every filter on, far field included (Diagnostic.cpp:718-996, FFTW stand-in):
    per slice the power, centroid, size, near- and far-field intensity and phase,
    far-field pointing and divergence; the window (Global/) values. Within 1e-12 of
    each column's scale (the far-field transforms round differently)."""
    import gen_golden
    d = golden("fft.npz")
    u = gen_golden.far_field(ng)
    want, want_g = d[f"ff{ng}_diag"], d[f"ff{ng}_global"]
    got = np.concatenate([oracle.diag_field(u, 6e-5, 1e-10, harm, first),
                          oracle.diag_field_fft(u, 6e-5, 1e-10, harm, first)], axis=1)
    for col in range(13):
        scale = np.abs(want[:, col]).max()
        if col in (9, 11):  # pointing, on the divergence's scale
            scale = np.abs(want[:, col + 1]).max()
        assert np.abs(got[:, col] - want[:, col]).max() <= 1e-12 * max(scale, 1e-300), col
    got_g = oracle.diag_global_field(u, 6e-5, 1e-10, harm, 1.0)
    for k in range(11):
        scale = abs(want_g[k]) if k not in (7, 9) else abs(want_g[k + 1])
        assert abs(got_g[k] - want_g[k]) <= 1e-12 * max(scale, 1e-300), k


@pytest.mark.parametrize("case", ["n25_s1", "n32_s2"])
def test_fft_solved_fields_far_field_matches_reference(oracle, case):
    """The far-field columns of the reference's solved FFT fields (fft.npz), from the
    oracle's diagnostics on the reference's own output fields."""
    d = golden("fft.npz")
    for k, hk in enumerate(d[f"{case}_harm"]):
        f = d[f"{case}_out_fields"][k]
        gm = float(d[f"{case}_gridmax"][k])
        first = int(d[f"{case}_out_first"][k])
        got = oracle.diag_field_fft(f, gm, 1e-10, int(hk), first)
        want = d[f"{case}_diag{k}"][:, 9:]
        for col in range(4):
            scale = np.abs(want[:, col | 1]).max()
            assert np.abs(got[:, col] - want[:, col]).max() <= 1e-12 * scale, (k, col)


@pytest.mark.parametrize("case", ["short", "long", "both", "steady"])
def test_space_charge_steps(oracle, case):
    """Space charge (&efield, EFieldSolver.cpp): the oracle's restatement against the
    reference run with its own EFieldSolver (tests/golden/spacecharge.npz): the
    short-range field of nz x (2 nphi + 1) modes on a radial grid grown from the
    slices' extent, the long-range loss over the window, and both."""
    d = golden("spacecharge.npz")
    g = lambda k: d[f"{case}_{k}"]
    gammaref, time_run, periodic = g("args")
    rmax, ngrid, nz, nphi, longrange = g("efield")
    oracle.set_efield(rmax, int(ngrid), int(nz), int(nphi), bool(longrange))
    try:
        part, fld, first, _ = oracle.run_steps(g("lat"), gammaref, g("part"), g("cur"), 1e-10, 1.0, g("harm"),
                                               g("gridmax"), g("fields"), g("first"), time_run=int(time_run),
                                               periodic=int(periodic), stages=7)
    finally:
        oracle.set_efield()
    if EXACT:
        assert np.array_equal(part, g("out_part"))
        assert np.array_equal(fld, g("out_fields"))
    else:
        assert np.allclose(part, g("out_part"), rtol=1e-12, atol=0)
        assert np.allclose(fld, g("out_fields"), rtol=1e-12, atol=1e-12 * np.abs(g("out_fields")).max())
    assert np.array_equal(first, g("out_first"))


def test_space_charge_grid_extent_carries_over(oracle):
    """The radial grid extent is EFieldSolver state: two runs of one step each, without
    a reset between them, equal one run of two steps."""
    d = golden("spacecharge.npz")
    g = lambda k: d[f"both_{k}"]
    gammaref, time_run, periodic = g("args")
    rmax, ngrid, nz, nphi, longrange = g("efield")
    lat = g("lat")
    kw = dict(time_run=int(time_run), periodic=int(periodic), stages=7)
    try:
        oracle.set_efield(rmax, int(ngrid), int(nz), int(nphi), bool(longrange))
        p2, f2, first2, _ = oracle.run_steps(lat[:2], gammaref, g("part"), g("cur"), 1e-10, 1.0, g("harm"),
                                             g("gridmax"), g("fields"), g("first"), **kw)
        oracle.set_efield(rmax, int(ngrid), int(nz), int(nphi), bool(longrange))
        p1, f1, first1, acc1 = oracle.run_steps(lat[:1], gammaref, g("part"), g("cur"), 1e-10, 1.0, g("harm"),
                                                g("gridmax"), g("fields"), g("first"), **kw)
        p1, f1, first1, _ = oracle.run_steps(lat[1:2], gammaref, p1, g("cur"), 1e-10, 1.0, g("harm"),
                                             g("gridmax"), f1, first1, accuslip=acc1, **kw)
    finally:
        oracle.set_efield()
    assert np.array_equal(p1, p2) and np.array_equal(f1, f2)


@pytest.mark.parametrize("case", ["s1", "s1_transient", "s3"])
def test_wake_steps(oracle, case):
    """Wakes (&wake, Collective.cpp): the oracle's restatement of the wake update and
    its application against the reference run with its own Collective
    (tests/golden/wakes.npz): windows of sample 1 and 3 with an external loss and the
    resistive, geometric and roughness wakes, and a transient wake."""
    d = golden("wakes.npz")
    g = lambda k: d[f"{case}_{k}"]
    gammaref, time_run, periodic, sample = g("args")
    ds, ztrans, radius, transient = g("wake_par")
    oracle.set_wake(g("wake_ext"), g("wake_res"), g("wake_geo"), g("wake_rou"), ds, ztrans, radius, bool(transient))
    try:
        part, fld, first, _ = oracle.run_steps(g("lat"), gammaref, g("part"), g("cur"), 1e-10, sample, g("harm"),
                                               g("gridmax"), g("fields"), g("first"), time_run=int(time_run),
                                               periodic=int(periodic), stages=7)
    finally:
        oracle.set_wake()
    if EXACT:
        assert np.array_equal(part, g("out_part"))
        assert np.array_equal(fld, g("out_fields"))
    else:
        assert np.allclose(part, g("out_part"), rtol=1e-12, atol=0)
        assert np.allclose(fld, g("out_fields"), rtol=1e-12, atol=1e-12 * np.abs(g("out_fields")).max())
    assert np.array_equal(first, g("out_first"))


@pytest.mark.parametrize("case", ["td", "steady"])
def test_chicane_steps(oracle, case):
    """A chicane between two undulator modules (TrackBeam::applyChicane, applyR56): the
    oracle against the reference run (tests/golden/chicane.npz)."""
    d = golden("chicane.npz")
    g = lambda k: d[f"{case}_{k}"]
    gammaref, time_run, periodic = g("args")
    oracle.set_chicanes(g("chic"))
    try:
        part, fld, first, _ = oracle.run_steps(g("lat"), gammaref, g("part"), g("cur"), 1e-10, 1.0, g("harm"),
                                               g("gridmax"), g("fields"), g("first"), time_run=int(time_run),
                                               periodic=int(periodic), stages=7)
    finally:
        oracle.set_chicanes()
    if EXACT:
        assert np.array_equal(part, g("out_part"))
        assert np.array_equal(fld, g("out_fields"))
    else:
        assert np.allclose(part, g("out_part"), rtol=1e-12, atol=0)
        assert np.allclose(fld, g("out_fields"), rtol=1e-12, atol=1e-12 * np.abs(g("out_fields")).max())
    assert np.array_equal(first, g("out_first"))


@pytest.mark.parametrize("case", ["every", "third"])
def test_one4one_sorting_steps(oracle, case):
    """One4one windows (slices of different particle counts) sorted after the push
    (Beam::sort, Sorting::globalSort / localSort for one rank): the oracle against the
    reference run (tests/golden/one4one.npz), particles in the reference's order."""
    d = golden("one4one.npz")
    g = lambda k: d[f"{case}_{k}"]
    gammaref, time_run, periodic, every = g("args")
    rmax, ngr, nz, nphi, lr = g("efield")
    oracle.set_counts(g("counts"), int(every))
    oracle.set_efield(rmax, int(ngr), int(nz), int(nphi), bool(lr))
    try:
        part, fld, first, _ = oracle.run_steps(g("lat"), gammaref, g("part"), g("cur"), 1e-10, 1.0, g("harm"),
                                               g("gridmax"), g("fields"), g("first"), time_run=int(time_run),
                                               periodic=int(periodic), stages=7)
        counts = oracle.get_counts(g("counts").size)
    finally:
        oracle.set_counts()
        oracle.set_efield()
    assert np.array_equal(counts, g("out_counts"))
    for i, n in enumerate(counts):
        if EXACT:
            assert np.array_equal(part[i, :n], g("out_part")[i, :n])
        else:
            assert np.allclose(part[i, :n], g("out_part")[i, :n], rtol=1e-12, atol=0)
    if EXACT:
        assert np.array_equal(fld, g("out_fields"))
    else:
        assert np.allclose(fld, g("out_fields"), rtol=1e-12, atol=1e-12 * np.abs(g("out_fields")).max())
    assert np.array_equal(first, g("out_first"))


def test_sort_drops_and_moves_like_the_reference(oracle):
    """orc_sort on its own: phases beyond the slice move, the window's ends drop,
    currents follow the counts (ce / slicelength per particle)."""
    ns, cap = 3, 8
    part = np.zeros((ns, cap, 6))
    counts = np.array([4, 3, 2], dtype=np.int32)
    th = [[0.5, 7.0, -0.25, 13.0], [1.0, -7.0, 20.0], [6.0, 6.5]]
    for i, t in enumerate(th):
        part[i, :len(t), 1] = t
        part[i, :len(t), 0] = 100 * i + np.arange(len(t))  # labels
    p, c, cur, lost = oracle.sort(part, counts, np.zeros(ns), 1e-10, 1.0)
    assert lost == 0
    two_pi = 2 * np.pi
    got = {i: sorted((round(p[i, k, 0]), round(p[i, k, 1], 9)) for k in range(c[i])) for i in range(ns)}
    # slice 0: 0.5 stays, 7.0 -> slice 1, -0.25 drops (s < 0), 13.0 -> slice 2;
    # slice 1: 1.0 stays, -7.0 drops (s < 0), 20.0 drops (s > 3 * 2 pi);
    # slice 2: 6.0 stays, 6.5 drops (s > 3 * 2 pi)
    assert got[0] == [(0, 0.5)]
    assert got[1] == sorted([(1, round(7.0 - two_pi, 9)), (100, 1.0)])
    assert got[2] == sorted([(3, round(13.0 - 2 * two_pi, 9)), (200, 6.0)])
    assert np.allclose(cur, c * 4.8032045e-11 / 1e-10)


@pytest.mark.parametrize("case", ["loss", "loss_helical", "spread"])
def test_incoherent_radiation_steps(oracle, case):
    """Incoherent synchrotron radiation (Incoherent::init / apply): the oracle's ran2
    stream and energy changes against the reference run (tests/golden/incoherent.npz)."""
    d = golden("incoherent.npz")
    seed, loss, spread, nbins = d[f"{case}_isr"]
    oracle.set_incoherent(int(seed), bool(loss), bool(spread), int(nbins))
    try:
        part, fld, _, _ = oracle.run_steps(d[f"{case}_lat"], 11357.8, d[f"{case}_part"], d["cur"], 1e-10, 1.0, [1],
                                           [6e-5], d["fields"], [0], time_run=1, stages=7)
    finally:
        oracle.set_incoherent()
    if EXACT:
        assert np.array_equal(part, d[f"{case}_out_part"])
        assert np.array_equal(fld, d[f"{case}_out_fields"])
    else:
        assert np.allclose(part, d[f"{case}_out_part"], rtol=1e-12, atol=0)
