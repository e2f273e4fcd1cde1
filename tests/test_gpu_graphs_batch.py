"""GPU tests of the captured-graph mode, the launch-shape autotuner and batched
ensembles of uneven runs: each must reproduce the plain direct-launch results.

The deposition adds with atomics, whose order varies from run to run: results of
two executions agree to rounding (1e-12 relative in FP64, 1e-5 in the mixed form),
not bit for bit.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel_err(a, b):
    scale = np.max(np.abs(b))
    return float(np.max(np.abs(np.asarray(a) - b)) / scale) if scale > 0 else float(np.max(np.abs(a - b)))


def window(ns, npart, ngrid, seed, taper=0.0, nwig=20):
    import g4gpu
    import g4cases as T
    cur = T.flat_top_current(ns, 1e-10, 1.0, 3000.0, ns * 1e-10 / 8)
    sp = T.slice_params(ns, 11357.8, 2.0, 0.4e-6, 15.0, currents=cur)
    beam = g4gpu.host_load_beam(sp, 0, npart, 4, seed, 1, 1e-10, 1.0)
    lat = T.undulator_lattice(1.7, 0.015, nwig, 2, 1e-10, 11357.8, quad_k1=1.5, quad_l=0.08, taper=taper)
    gh = g4gpu.host_gauss_hermite(T.gauss_field_par(1e-10, 1e4, 25e-6), 1e-4, ngrid)
    fld = np.stack([gh * (1 + 0.01 * k) for k in range(ns)])
    return lat, beam, cur, fld


def make(lat, beam, cur, fld, precision, solver=0, graph=False):
    import g4gpu
    ns, npart = beam.shape[0], beam.shape[1]
    ngrid = int(round(np.sqrt(fld.shape[1])))
    cfg = g4gpu.Config(nslice=ns, npart=npart, ngrid=ngrid, gridmax=1e-4, lambda0=1e-10, sample=1.0,
                       gammaref=11357.8, precision=precision, solver=solver, time_run=1)
    h = g4gpu.Handle(cfg)
    h.set_lattice(lat)
    h.load_beam(beam, cur)
    h.load_field(0, fld)
    h.set_graph_mode(graph)
    return h


@pytest.mark.parametrize("precision,tol", [(0, 1e-12), (1, 1e-5)])
def test_graph_mode_matches_direct_launches(lib, precision, tol):
    lat, beam, cur, fld = window(8, 256, 41, 3)
    with make(lat, beam, cur, fld, precision) as h:
        h.run(0, lat.shape[0])
        p0 = h.get_beam()
        f0, first0, acc0 = h.get_field(0)
    with make(lat, beam, cur, fld, precision, graph=True) as h:
        for rep in range(2):  # capture, then replay from the same starting state
            h.load_beam(beam, cur)
            h.load_field(0, fld)
            h.run(0, 10)
            h.run(10, lat.shape[0] - 10)
            p1 = h.get_beam()
            f1, first1, acc1 = h.get_field(0)
            assert first1 == first0 and acc1 == acc0
            assert rel_err(f1, f0) < tol
            for col in (0, 2, 3, 4, 5):
                assert rel_err(p1[..., col], p0[..., col]) < tol
            assert np.max(np.abs(p1[..., 1] - p0[..., 1])) < 1e-6
        st = h.kernel_stats()
        assert st["push"][0] == 2 * lat.shape[0]


@pytest.mark.parametrize("precision", [0, 1])
def test_autotune_keeps_results(lib, precision):
    lat, beam, cur, fld = window(16, 512, 61, 5)
    with make(lat, beam, cur, fld, precision) as h:
        pb, ft, fk = h.autotune()
        assert pb in (128, 256, 512)
        assert ft % 32 == 0 and 2 * 61 <= ft <= 1024
        assert fk in (0, 1, 2) and (precision == 1 or fk == 0)
        # the tuning steps are undone
        p = h.get_beam()
        assert np.array_equal(p, beam) if precision == 0 else rel_err(p, beam) < 1e-6
        h.run(0, lat.shape[0])
        bd, fd = h.diag(1)
    with make(lat, beam, cur, fld, precision) as h:
        h.run(0, lat.shape[0])
        bd0, fd0 = h.diag(1)
    assert rel_err(fd[0][:, 0], fd0[0][:, 0]) < (1e-10 if precision == 0 else 1e-4)


def test_batch_of_uneven_runs_matches_single_runs(lib):
    """Ensemble members with different slice counts, particle counts, grids (one too
    large for the shared-memory field kernel) and tapers."""
    import g4gpu
    specs = [(6, 256, 41, 1, 0.0, 0), (11, 512, 51, 2, -0.02, 0), (4, 128, 181, 3, -0.01, 0),
             (7, 256, 45, 4, 0.0, 1)]
    cases = []
    cfgs = []
    for ns, npart, ngrid, seed, taper, solver in specs:
        lat, beam, cur, fld = window(ns, npart, ngrid, seed, taper=taper, nwig=12)
        cases.append((lat, beam, cur, fld, solver))
        cfgs.append(g4gpu.Config(nslice=ns, npart=npart, ngrid=ngrid, gridmax=1e-4, lambda0=1e-10, sample=1.0,
                                 gammaref=11357.8, precision=1, solver=solver, time_run=1))
    with g4gpu.Batch(cfgs) as b:
        for m, (lat, beam, cur, fld, solver) in zip(b.members, cases):
            m.set_lattice(lat)
        n = max(c[0].shape[0] for c in cases)
        # twice from the same state: the ensemble's step ranges are captured as one graph
        # each the first time and replayed the second
        for rep in range(2):
            for m, (lat, beam, cur, fld, solver) in zip(b.members, cases):
                m.load_beam(beam, cur)
                m.load_field(0, fld)
            b.run(0, 9)
            b.run(9, n - 9)
            b.synchronize()
            got = [m.diag(1) for m in b.members]
            if rep == 0:
                first = got
        for (bd0, fd0), (bd1, fd1) in zip(first, got):
            assert rel_err(fd1[0][:, 0], fd0[0][:, 0]) < 1e-5
        for m, (lat, _, _, _, _) in zip(b.members, cases):
            assert m.kernel_stats()["push"][0] == 2 * lat.shape[0]
    for (lat, beam, cur, fld, solver), (bd, fd) in zip(cases, got):
        with make(lat, beam, cur, fld, 1, solver=solver) as h:
            h.run(0, lat.shape[0])
            bd0, fd0 = h.diag(1)
        assert rel_err(fd[0][:, 0], fd0[0][:, 0]) < 1e-4
        assert np.max(np.abs(bd[:, 24] - bd0[:, 24])) < 1e-4


@pytest.mark.parametrize("ng", [51, 151, 201, 255])
def test_cluster_pair_field_kernel_matches_single_cta(lib, ng):
    """The mixed form's field step on a cluster of CTAs per slice (rows split into
    bands, column solves across the bands through distributed shared memory): a pair
    against the one-CTA-per-slice kernel (ngrid <= 168), and the pair (ngrid 201) or a
    cluster of three (ngrid 255), the default for grids too large for one CTA, against
    the FP64 form: a lasing window over whole undulator steps with slippage."""
    import g4gpu
    import g4cases as T
    ns, npart = 24, 1024
    lat = T.undulator_lattice(1.7, 0.015, 30, 1, 1e-10, 17081.0)
    cur = np.full(ns, 3000.0)
    beam = g4gpu.host_load_beam(T.slice_params(ns, 17081.0, 2.0, 0.4e-6, 15.0, currents=cur), 0, npart, 4, 5, 1,
                                1e-10, 1.0)
    seed = g4gpu.host_gauss_hermite(T.gauss_field_par(1e-10, 1e5, 30e-6), 1e-4, ng)
    fld = np.repeat(seed[None, :], ns, axis=0)
    out = []
    for fk in (1, 0):
        cfg = g4gpu.Config(nslice=ns, npart=npart, ngrid=ng, gridmax=1e-4, lambda0=1e-10, sample=1.0,
                           gammaref=17081.0, precision=1, time_run=1)
        with g4gpu.Handle(cfg) as h:
            h.set_lattice(lat)
            h.load_beam(beam, cur)
            h.load_field(0, fld, first=7)
            if ng <= 168:
                h.set_launch_shapes(256, max(512, (2 * ng + 31) // 32 * 32), fk)
            elif fk == 0:
                continue
            h.run(0, lat.shape[0])
            out.append((h.diag(1), h.get_field(0)[0], h.get_beam()))
    if ng > 168:
        # the pair against the FP64 form
        cfgp = g4gpu.Config(nslice=ns, npart=npart, ngrid=ng, gridmax=1e-4, lambda0=1e-10, sample=1.0,
                            gammaref=17081.0, precision=0, time_run=1)
        with g4gpu.Handle(cfgp) as h:
            h.set_lattice(lat)
            h.load_beam(beam, cur)
            h.load_field(0, fld, first=7)
            h.run(0, lat.shape[0])
            out.append((h.diag(1), h.get_field(0)[0], h.get_beam()))
        tol = 1e-2
    else:
        tol = 1e-4
    (b1, f1), F1, P1 = out[0]
    (b0, f0), F0, P0 = out[1]
    assert rel_err(f1[0][:, 0], f0[0][:, 0]) < tol
    assert rel_err(F1, F0) < (tol if ng <= 168 else 1e-2)
    assert np.max(np.abs(b1[:, 24] - b0[:, 24])) <= tol * np.max(np.abs(b0[:, 24])) + 1e-4



def test_ensemble_members_match_oracle(lib, oracle):
    """Members shaped like the uneven ensemble's draws, run as one batch in the mixed
    form (captured graphs, launch shapes from the autotuner), each against the FP64
    oracle (bit-exact with the reference): linear aw tapers over four modules, ngrid
    201 (cluster-pair field kernel) and 255 (a cluster of three), npart 2048 and 16384,
    a 1 kW seed over shot noise, periodic windows (at 2.26 slices of slippage per step
    a zero-filled window of a few slices would be emptied within two steps). Slice
    power within 1 % of the largest slice power, bunching within 1 % of the largest
    plus 1e-3 (far below the shot-noise level 1/sqrt(npart) of these beams)."""
    import g4gpu
    import g4cases as T
    specs = [(8, 2048, 201, 11, -0.015), (4, 16384, 255, 12, -0.007), (6, 4096, 101, 13, -0.02)]
    cases, cfgs = [], []
    for ns, npart, ngrid, seed, taper in specs:
        cur = T.flat_top_current(ns, 1e-10, 1.0, 3000.0, ns * 1e-10 / 8)
        sp = T.slice_params(ns, 11357.8, 2.0, 0.4e-6, 15.0, currents=cur)
        beam = g4gpu.host_load_beam(sp, 0, npart, 4, seed, 1, 1e-10, 1.0)
        lat = T.undulator_lattice(1.7, 0.015, 10, 4, 1e-10, 11357.8, quad_k1=1.5, quad_l=0.08, taper=taper)
        gh = g4gpu.host_gauss_hermite(T.gauss_field_par(1e-10, 1e3, 30e-6), 1e-4, ngrid)
        fld = np.repeat(gh[None, :], ns, axis=0)
        cases.append((lat, beam, cur, fld))
        cfgs.append(g4gpu.Config(nslice=ns, npart=npart, ngrid=ngrid, gridmax=1e-4, lambda0=1e-10, sample=1.0,
                                 gammaref=11357.8, precision=1, time_run=1, periodic=1))
    with g4gpu.Batch(cfgs) as b:
        for m, (lat, beam, cur, fld) in zip(b.members, cases):
            m.set_lattice(lat)
            m.load_beam(beam, cur)
            m.load_field(0, fld)
            m.autotune()
        b.run(0, max(c[0].shape[0] for c in cases))
        b.synchronize()
        got = [m.diag(1) for m in b.members]
    for (lat, beam, cur, fld), (bd, fd), (ns, npart, ngrid, _, taper) in zip(cases, got, specs):
        assert abs(lat[-1, 0] / lat[0, 0] - 1 - taper) < 1e-12  # the taper spans the lattice
        rp, rf, rfirst, _ = oracle.run_steps(lat, 11357.8, beam, cur, 1e-10, 1.0, [1], [1e-4], fld[None], [0],
                                             nthreads=8, periodic=1)
        of = oracle.diag_field(rf[0], 1e-4, 1e-10, 1, int(rfirst[0]))
        ob = oracle.diag_beam(rp, 1)
        assert of[:, 0].max() > 0
        assert rel_err(fd[0][:, 0], of[:, 0]) < 1e-2, (ngrid, npart)
        assert np.max(np.abs(bd[:, 24] - ob[:, 24])) <= 1e-2 * np.max(ob[:, 24]) + 1e-3, (ngrid, npart)


@pytest.mark.parametrize("ng,npart", [(51, 1024), (151, 2048), (101, 1000)])
def test_whole_step_kernel_matches_push_and_field_kernels(lib, oracle, ng, npart):
    """The whole step of a slice in one kernel (launch shape field_kernel 2: push,
    deposition and ADI in one CTA) against the push kernel followed by the fused field
    kernel (field_kernel 0), at every CTA size the autotuner tries (each with its own
    particles per lane), over a lasing window with slippage; and against the FP64
    oracle within the mixed form's 1 %. npart 1000 leaves a part-filled last round of
    every warp. The run_diag records the whole-step kernel forms itself (the beam's and
    the field's) agree with g4gpu_diag after the same steps."""
    import g4gpu
    import g4cases as T
    ns = 24
    lat = T.undulator_lattice(1.7, 0.015, 30, 1, 1e-10, 17081.0)
    cur = np.full(ns, 3000.0)
    beam = g4gpu.host_load_beam(T.slice_params(ns, 17081.0, 2.0, 0.4e-6, 15.0, currents=cur), 0, npart, 4, 5, 1,
                                1e-10, 1.0)
    seed = g4gpu.host_gauss_hermite(T.gauss_field_par(1e-10, 1e5, 30e-6), 1e-4, ng)
    fld = np.repeat(seed[None, :], ns, axis=0)
    cfg = g4gpu.Config(nslice=ns, npart=npart, ngrid=ng, gridmax=1e-4, lambda0=1e-10, sample=1.0,
                       gammaref=17081.0, precision=1, time_run=1)
    lo = (2 * ng + 31) // 32 * 32
    results = {}
    for fk, ft in [(0, 1024)] + [(2, t) for t in sorted({lo, 512, 768, 1024}) if t >= lo]:
        with g4gpu.Handle(cfg) as h:
            h.set_lattice(lat)
            h.load_beam(beam, cur)
            h.load_field(0, fld, first=5)
            h.set_launch_shapes(256, ft, fk)
            h.run(0, lat.shape[0])
            st = h.kernel_stats()
            if fk == 2:
                assert st["step"][0] == lat.shape[0] and st["push"][0] == 0
            results[(fk, ft)] = (h.diag(1), h.get_field(0)[0], h.get_beam())
            # run_diag of three more steps: records formed by the whole-step kernel
            if fk == 2:
                h.load_beam(beam, cur)
                h.load_field(0, fld, first=5)
                bd3, fd3 = h.run_diag(0, 3, 1)
                b3, f3 = h.diag(1)
                assert rel_err(fd3[-1][0][:, 0], f3[0][:, 0]) < 1e-5
                for col in (0, 1, 2, 3, 24):
                    assert np.max(np.abs(bd3[-1][:, col] - b3[:, col])) <= 1e-5 * np.max(np.abs(b3[:, col])) + 1e-9
    (b0, f0), F0, P0 = results[(0, 1024)]
    for key, ((b1, f1), F1, P1) in results.items():
        assert rel_err(f1[0][:, 0], f0[0][:, 0]) < 1e-4, key
        assert rel_err(F1, F0) < 1e-4, key
        assert np.max(np.abs(b1[:, 24] - b0[:, 24])) <= 1e-4 * np.max(np.abs(b0[:, 24])) + 1e-6, key
    rp, rf, rfirst, _ = oracle.run_steps(lat, 17081.0, beam, cur, 1e-10, 1.0, [1], [1e-4], fld[None], [5],
                                         nthreads=8)
    of = oracle.diag_field(rf[0], 1e-4, 1e-10, 1, int(rfirst[0]))
    (b2, f2), _, _ = results[(2, 1024)]
    assert rel_err(f2[0][:, 0], of[:, 0]) < 1e-2
