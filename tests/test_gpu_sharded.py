"""A time window sharded over ranks on one GPU: two and three handles, each holding
a contiguous block of the window's slices (sharded.block, GenTime.cpp:74-77), driven
in lockstep by sharded.LocalRing, which moves the boundary slices of every slippage
shift between the ranks' buffers (g4gpu_shift_out / g4gpu_shift_in, the exchange of
Control::applySlippage, Control.cpp:183-275). The blocks, put together, must
reproduce the single handle that holds the whole window: every slice's step is the
same arithmetic, so only the deposition's atomic summation order differs (1e-12 of
the largest value in FP64, 1e-5 in the mixed form)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel_err(a, b):
    scale = np.max(np.abs(b))
    return float(np.max(np.abs(np.asarray(a) - b)) / scale) if scale > 0 else float(np.max(np.abs(a - b)))


@pytest.mark.parametrize("precision,tol", [(0, 1e-12), (1, 1e-5)])
@pytest.mark.parametrize("nrank,periodic", [(2, 0), (2, 1), (3, 0)])
def test_sharded_window_matches_whole_window(lib, precision, tol, nrank, periodic):
    import g4gpu
    import g4cases as T
    import sharded
    ns, npart, ng = 18, 256, 41
    lat = T.undulator_lattice(1.7, 0.015, 8, 2, 1e-10, 11357.8, quad_k1=1.5, quad_l=0.08)
    cur = T.flat_top_current(ns, 1e-10, 1.0, 3000.0, ns * 1e-10 / 8)
    beam = g4gpu.host_load_beam(T.slice_params(ns, 11357.8, 2.0, 0.4e-6, 15.0, currents=cur), 0, npart, 4, 7, 1,
                                1e-10, 1.0)
    seed = g4gpu.host_gauss_hermite(T.gauss_field_par(1e-10, 1e5, 20e-6), 6e-5, ng)
    fld = np.stack([seed * (1 + 0.1j * k) for k in range(ns)])

    def config(n):
        return g4gpu.Config(nslice=n, npart=npart, ngrid=ng, gridmax=6e-5, lambda0=1e-10, sample=1.0,
                            gammaref=11357.8, precision=precision, time_run=1, periodic=periodic)

    with g4gpu.Handle(config(ns)) as h:
        h.set_lattice(lat)
        h.load_beam(beam, cur)
        h.load_field(0, fld)
        h.run(0, lat.shape[0])
        want_p = h.get_beam()
        f, first, acc = h.get_field(0)
        want_f = f[(np.arange(ns) + first) % ns]
    handles = []
    try:
        for r in range(nrank):
            s0, n = sharded.block(ns, r, nrank)
            hr = g4gpu.Handle(config(n))
            hr.set_lattice(lat)
            hr.load_beam(beam[s0:s0 + n], cur[s0:s0 + n])
            hr.load_field(0, fld[s0:s0 + n])
            handles.append(hr)
        ring = sharded.LocalRing(handles, periodic)
        for i in range(lat.shape[0]):
            ring.step(i, lat[i, T.C["slip"]], 1)
        got_p = np.concatenate([hr.get_beam() for hr in handles])
        parts = []
        for hr in handles:
            f, first, acc_r = hr.get_field(0)
            assert acc_r == acc
            parts.append(f[(np.arange(f.shape[0]) + first) % f.shape[0]])
        got_f = np.concatenate(parts)
    finally:
        for hr in handles:
            hr.close()
    assert np.abs(want_f).max() > 0
    assert rel_err(got_f, want_f) < tol
    for col in range(6):
        assert rel_err(got_p[..., col], want_p[..., col]) < tol, col


def test_shift_in_needs_a_shift_out(lib):
    import g4gpu
    cfg = g4gpu.Config(nslice=4, npart=32, ngrid=11, gridmax=6e-5, lambda0=1e-10, sample=1.0,
                       gammaref=11357.8, precision=1, time_run=1)
    with g4gpu.Handle(cfg) as h:
        with pytest.raises(g4gpu.G4Error) as e:
            h.shift_in(0, 0)
        assert e.value.code == 3
        h.shift_out(0, 1, 0)
        with pytest.raises(g4gpu.G4Error) as e:
            h.shift_out(0, 1, 0)
        assert e.value.code == 3
        h.shift_in(0, 0)
