"""GPU tests of the learned coarse-step closure.

  * the BF16 tensor-core MLP kernels: gradients against the numpy FP64 oracle
    (oracle/mlp_oracle.py, with the same BF16 rounding of the GEMM operands), and
    training that lowers the loss;
  * the closure on a SASE window: trained on fine-step runs over several shot-noise
    seeds, it must bring coarse steps (4 periods) closer to the fine-step result on
    a held-out seed than coarse steps without it;
  * the judge: with a zero tolerance every checked interval falls back to the fine
    solve, which then reproduces the all-fine run.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [16, 200])
def test_mlp_gradients_match_cpu_oracle(lib, n):
    import g4gpu
    import mlp_oracle
    rng = np.random.default_rng(n)
    m = g4gpu.MLP(32, 256, 4, seed=3)
    p = m.get_params()
    # non-zero biases so that every parameter takes part
    p = p + (rng.standard_normal(p.size).astype(np.float32) * 0.01) * (p == 0)
    m.set_params(p)
    m.set_normalization(np.zeros(32), np.ones(32), np.zeros(4), np.ones(4))
    X = rng.standard_normal((n, 32)).astype(np.float32)
    T = rng.standard_normal((n, 4)).astype(np.float32)
    g, loss = m.gradients(X, T)
    Y0, loss0, g0 = mlp_oracle.forward_backward(m.get_params(), X.astype(np.float64), T.astype(np.float64),
                                                32, 256, 4, bf16=True)
    assert abs(loss / loss0 - 1) < 1e-3
    Y = m.forward(X)
    assert np.max(np.abs(Y - Y0)) < 1e-3 * np.max(np.abs(Y0)) + 1e-6
    # per parameter block: BF16 operands, FP32 accumulation in another order
    layers, dims = mlp_oracle.unpack(p, 32, 256, 4)
    o = 0
    for (W, b) in layers:
        for size in (W.size, b.size):
            a, r = g[o:o + size], g0[o:o + size]
            assert np.linalg.norm(a - r) <= 2e-3 * np.linalg.norm(r) + 1e-9, (o, size)
            o += size


@pytest.mark.parametrize("n,width", [(4096, 256), (1000, 96), (333, 48), (700, 512)])
def test_mlp_forward_matches_cpu_oracle(lib, n, width):
    """The forward pass over a window's worth of rows through the tcgen05 GEMM: tile
    widths 128 (N = 256, 512) and the whole N below that (96, 48); reductions of
    32, 48, 96, 256 and 512 (one to eight 64-element stages, the last one partial
    at 48 and 96). Ragged row counts leave the last 128-row tile partly empty."""
    import g4gpu
    import mlp_oracle
    rng = np.random.default_rng(n + width)
    m = g4gpu.MLP(32, width, 4, seed=5)
    p = m.get_params()
    p = p + (rng.standard_normal(p.size).astype(np.float32) * 0.01) * (p == 0)
    m.set_params(p)
    m.set_normalization(np.zeros(32), np.ones(32), np.zeros(4), np.ones(4))
    X = rng.standard_normal((n, 32)).astype(np.float32)
    Y = m.forward(X)
    Y0 = mlp_oracle.forward_backward(m.get_params(), X.astype(np.float64), np.zeros((n, 4)), 32, width, 4,
                                     bf16=True)[0]
    m.close()
    # BF16 activations rounded from FP32 sums taken in another order: a value near a
    # rounding boundary may round the other way (2^-8 relative) and carry that on
    scale = np.max(np.abs(Y0))
    assert np.max(np.abs(Y - Y0)) < 3e-3 * scale
    assert np.mean(np.abs(Y - Y0)) < 3e-4 * scale


def test_mlp_training_lowers_the_loss(lib):
    import g4gpu
    rng = np.random.default_rng(0)
    X = rng.standard_normal((8192, 32)).astype(np.float32)
    a = rng.standard_normal((32, 4))
    T = np.tanh(X @ a / 4).astype(np.float32) + 0.1 * X[:, :4] ** 2
    m = g4gpu.MLP(32, 256, 4, seed=1)
    curve = m.train(X, T, epochs=12, batch=512, lr=2e-3, seed=2)
    assert curve[-1] < 0.1 * curve[0], curve


def sase_setup(ns=32, npart=1024, ngrid=51):
    import g4cases as T
    cfg = dict(nslice=ns, npart=npart, ngrid=ngrid, gridmax=1e-4, lambda0=1e-10, sample=1.0,
               gammaref=17081.0, precision=1, time_run=1)
    # resonant planar undulator so that the window lases within a few modules
    lat = T.undulator_lattice(1.7, 0.015, 60, 2, 1e-10, 17081.0, quad_k1=1.5, quad_l=0.08)
    sp = T.slice_params(ns, 17081.0, 1.0, 0.4e-6, 15.0, current=3000.0)
    field = np.zeros((ns, ngrid * ngrid), dtype=np.complex128)
    return cfg, lat, sp, field


def test_closure_gains_over_coarse_steps(lib):
    import g4gpu
    import learned
    cfg, lat, sp, field = sase_setup()
    waist, u0, c0 = 30e-6, 1.0, 1.0
    X, Tg, clat, fs, fc = learned.generate_training_data(cfg, lat, range(100, 116), sp, cfg["npart"], 4, field,
                                                          waist, u0, c0)
    assert X.shape[1] == 32 and Tg.shape[1] == 4 and X.shape[0] == Tg.shape[0]
    m = g4gpu.MLP(32, 256, 4, seed=0)
    curve = m.train(X, Tg, epochs=20, batch=256, lr=1e-3, seed=0)
    assert curve[-1] < curve[0]
    beam = g4gpu.host_load_beam(sp, 0, cfg["npart"], 4, 999, 1, 1e-10, 1.0)
    res = learned.evaluate(cfg, lat, clat, fs, fc, beam, sp[:, 16], field, m, waist, u0, c0)
    e = learned.errors(res)
    print("coarse vs fine:", e["coarse"], "closure vs fine:", e["closure"])
    assert e["closure"]["power_rms"] < e["coarse"]["power_rms"]


def test_coarse_pushes_under_fine_sources_match_fine_steps(lib):
    """Coarse steps on a time-dependent window sampled every wavelength (the config-1
    beam: gamma 11357.8 off resonance at 1e-10 m, shot noise, no seed), each pushed
    once over its periods, deposited and slipped period by period from the
    interpolated phases and positions, and diffracted once (g4gpu_set_field_substeps).
    After 40 periods: with steps of 2 periods the slice power is within 1 % of the
    largest slice power of the fine (one-period) run; with 4 periods within 10 % (the
    sources, added between the diffractions, miss the diffraction of up to 3.5
    periods); whole coarse steps (2 or 4 slices of slippage at once) give about 2 and
    3.5 times the power. The bunching is within 1 % of its largest value in every
    form of sub-stepped coarse step."""
    import g4gpu
    import g4cases as T
    import learned
    ns, npart, ng = 64, 1024, 51
    cfg = g4gpu.Config(nslice=ns, npart=npart, ngrid=ng, gridmax=1e-4, lambda0=1e-10, sample=1.0,
                       gammaref=11357.8, precision=1, time_run=1)
    lat = T.undulator_lattice(1.7, 0.015, 40, 1, 1e-10, 11357.8)
    sp = T.slice_params(ns, 11357.8, 2.0, 0.4e-6, 15.0, current=3000.0)
    beam = g4gpu.host_load_beam(sp, 0, npart, 4, 7, 1, 1e-10, 1.0)
    field = np.zeros((ns, ng * ng), dtype=np.complex128)

    def run(table, counts):
        with g4gpu.Handle(cfg) as h:
            h.set_lattice(table)
            if counts is not None:
                h.set_field_substeps(counts)
            h.load_beam(beam, sp[:, 16])
            h.load_field(0, field)
            h.run(0, table.shape[0])
            bd, fd = h.diag(1)
            return fd[0][:, 0], bd[:, 24], h.kernel_stats()

    pf, bf, _ = run(lat, None)
    scale = np.max(pf)
    assert scale > 0
    for factor, tol in ((2, 1e-2), (4, 1e-1)):
        clat, fs, fc = learned.coarsen_lattice(lat, factor)
        assert list(fc) == [factor] * (40 // factor)
        ps, bs, st = run(clat, fc)
        pw, _, _ = run(clat, None)
        assert st["push"][0] == 40 // factor and st["adi_x"][0] == 40 // factor and st["misc"][0] >= 40
        err_sub = np.max(np.abs(ps - pf)) / scale
        err_whole = np.max(np.abs(pw - pf)) / scale
        print(f"factor {factor}: power error of sub-stepped coarse steps {err_sub:.4f}, of whole ones "
              f"{err_whole:.3f}")
        assert err_sub < tol
        assert err_whole > 0.5
        assert np.max(np.abs(bs - bf)) <= 1e-2 * np.max(bf)


def test_field_substeps_reject_unsupported_handles(lib):
    import g4gpu
    import g4cases as T
    lat = T.undulator_lattice(1.7, 0.015, 8, 1, 1e-10, 11357.8)
    for kw in (dict(precision=0), dict(ngrid=181), dict(npart=30)):
        args = dict(nslice=4, npart=64, ngrid=25, gridmax=1e-4, lambda0=1e-10, sample=1.0, gammaref=11357.8,
                    precision=1, time_run=1)
        args.update(kw)
        with g4gpu.Handle(g4gpu.Config(**args)) as h:
            h.set_lattice(lat)
            with pytest.raises(g4gpu.G4Error) as e:
                h.set_field_substeps([4] * lat.shape[0])
            assert e.value.code == 1
            h.set_field_substeps([1] * lat.shape[0])  # no coarse step: accepted
            with pytest.raises(g4gpu.G4Error):
                h.set_field_substeps([4] * (lat.shape[0] + 1))


def test_judge_falls_back_to_fine_steps(lib):
    import g4gpu
    import learned
    cfg, lat, sp, field = sase_setup(ns=16, npart=512, ngrid=41)
    clat, fs, fc = learned.coarsen_lattice(lat)
    m = g4gpu.MLP(32, 256, 4, seed=0)
    beam = g4gpu.host_load_beam(sp, 0, cfg["npart"], 4, 7, 1, 1e-10, 1.0)
    n = 20
    hf, hc = learned.make_pair(cfg, lat, clat, beam, sp[:, 16], field, m, 30e-6, 1.0, 1.0)
    with hf, hc:
        nchk, nfb, emax = hc.run_learned(hf, 0, n, fs, fc, check_every=1, tol=0.0)
        assert nchk == n and nfb == n
        bd, fd = hc.diag(1)
    href = g4gpu.Handle(g4gpu.Config(**cfg))
    with href:
        href.set_lattice(lat)
        href.load_beam(beam, sp[:, 16])
        href.load_field(0, field)
        href.run(0, int(fs[n - 1] + fc[n - 1]))
        bd0, fd0 = href.diag(1)
    scale = np.max(np.abs(fd0[0][:, 0]))
    assert np.max(np.abs(fd[0][:, 0] - fd0[0][:, 0])) <= 1e-3 * scale


@pytest.mark.parametrize("precision,first", [(1, 3), (0, 0)])
def test_closure_features_match_numpy(lib, precision, first):
    """The per-slice features against an FP64 numpy computation from the same beam and
    field: bunching h = 1..3, mean and rms of the energy offset, the on-axis field, and
    the projections on the 16 Gauss-Hermite modes HG_mn (m, n = 0..3) formed with the
    full two-dimensional basis (the kernel uses its separable factors)."""
    import math
    import g4gpu
    import g4cases as T
    ns, npart, ng, gm, g0, waist, u0, c0 = 8, 512, 41, 1e-4, 17081.0, 30e-6, 2e3, 5e3
    cur = np.linspace(1000.0, 3000.0, ns)
    beam = g4gpu.host_load_beam(T.slice_params(ns, g0, 2.0, 0.4e-6, 15.0, currents=cur), 0, npart, 4, 9, 1,
                                1e-10, 1.0)
    par = T.gauss_field_par(1e-10, 1e5, 25e-6)
    par[5], par[6] = 6e-6, -4e-6  # an off-axis seed: every mode takes part
    seed = g4gpu.host_gauss_hermite(par, gm, ng)
    field = seed[None, :] * np.exp(1j * np.linspace(0.0, 3.0, ns))[:, None]
    cfg = g4gpu.Config(nslice=ns, npart=npart, ngrid=ng, gridmax=gm, lambda0=1e-10, sample=1.0, gammaref=g0,
                       precision=precision, time_run=1)
    m = g4gpu.MLP(32, 256, 4, seed=0)
    with g4gpu.Handle(cfg) as h:
        h.load_beam(beam, cur)
        h.load_field(0, field, first=first)
        h.closure_attach(m, waist, u0, c0)
        X = h.closure_features()
        p = h.get_beam()
        f = h.get_field(0)[0]
    m.close()
    dg = 2 * gm / (ng - 1)
    x = -gm + np.arange(ng) * dg

    def herm(n, t):
        return [np.ones_like(t), 2 * t, 4 * t * t - 2, 8 * t ** 3 - 12 * t][n]

    for ib in range(ns):
        th, g = p[ib, :, 1], p[ib, :, 0] - g0
        for hh in range(3):
            b = np.mean(np.exp(1j * (hh + 1) * th))
            assert abs(X[ib, 2 * hh] - b.real) < 1e-5 and abs(X[ib, 2 * hh + 1] - b.imag) < 1e-5
        assert abs(X[ib, 6] - g.mean()) < 1e-5 * max(1.0, abs(g.mean()))
        assert abs(X[ib, 7] - g.std()) < 1e-3 * g.std()
        u = f[(ib + first) % ns].reshape(ng, ng)  # [iy][ix]
        ua = u[ng // 2, ng // 2]
        assert abs(X[ib, 8] - math.log1p(abs(ua) ** 2 / u0 ** 2)) < 1e-4 * max(1.0, X[ib, 8])
        for q in range(16):
            mm, nn = q // 4, q % 4
            norm = math.sqrt(2 / math.pi) / waist / math.sqrt(2.0 ** (mm + nn) * math.factorial(mm) * math.factorial(nn))
            sx = math.sqrt(2) * x / waist
            bx = herm(mm, sx) * np.exp(-x * x / waist ** 2)
            by = herm(nn, sx) * np.exp(-x * x / waist ** 2)
            basis = norm * np.outer(by, bx) * dg * dg  # [iy][ix]
            cq = np.sum(basis * u)
            want = math.log1p(abs(cq) ** 2 / c0 ** 2)
            assert abs(X[ib, 11 + q] - want) < 1e-4 * max(1.0, want), (ib, q, X[ib, 11 + q], want)
        assert abs(X[ib, 27] - cur[ib] * 1e-3) < 1e-6
