"""The single-precision ADI field step that allocates no device memory
(g4gpu_adi_advance_noalloc), called through the C ABI.

  * against the handle's own step (g4gpu_run, mixed form, field stage) on two calls
    in a row, with the source of an undulator step and with none on a drift;
  * against the oracle's FP64 ADI step (FieldSolverADI.cpp:9-122) on a window of
    more slices than CTAs, so that each CTA reuses its scratch slot, on two calls in
    a row;
  * sizes beyond its limits and bad pointers are rejected with G4GPU_ERR_ARG.

The file name sorts last, so that in a full run the scratch array already holds
what earlier calls left; the tests pass alone in a fresh process too.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NS, NPART, NG, GRIDMAX, LAMBDA0, GAMMA0 = 12, 1024, 51, 1e-4, 1e-10, 11357.8
# same bound for every comparison: |difference| <= TOL * max |field|; the FP32 step
# against the FP64 oracle differs by ~1e-6 of that
TOL = 1e-4


def setup_window(first):
    import g4cases as T
    import g4gpu
    lat = T.undulator_lattice(1.7, 0.015, 4, 2, LAMBDA0, GAMMA0, quad_k1=1.5, quad_l=0.08)
    sp = T.slice_params(NS, GAMMA0, 2.0, 0.4e-6, 15.0, current=3000.0)
    beam = g4gpu.host_load_beam(sp, 0, NPART, 4, 11, 1, LAMBDA0, 1.0)
    seed = g4gpu.host_gauss_hermite(T.gauss_field_par(LAMBDA0, 1e3, 30e-6), GRIDMAX, NG)
    phases = np.exp(1j * np.linspace(0.0, 2.0, NS))
    field = (seed[None, :] * phases[:, None]).astype(np.complex128)
    cfg = g4gpu.Config(nslice=NS, npart=NPART, ngrid=NG, gridmax=GRIDMAX, lambda0=LAMBDA0,
                       sample=1.0, gammaref=GAMMA0, precision=g4gpu.MIXED, time_run=1)
    h = g4gpu.Handle(cfg)
    h.set_lattice(lat)
    h.load_beam(beam, sp[:, 16])
    h.load_field(0, field, first=first)
    return h, lat, sp[:, 16]


def step_args(lat, istep):
    dgrid = 2 * GRIDMAX / (NG - 1)
    xks = 4.0 * math.asin(1) / LAMBDA0
    return float(lat[istep, 13]), dgrid, xks


def to_device(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.complex64)).to("cuda")


def close(got, want):
    return np.max(np.abs(got - want)) <= TOL * np.max(np.abs(want))


def test_noalloc_matches_handle_step_with_source(lib, oracle):
    import torch
    import g4gpu
    first = 5
    h, lat, cur = setup_window(first)
    with h:
        f_dev = to_device(torch, h.get_field(0)[0])
        for istep in (0, 1):  # two undulator steps: two calls in a row
            h.run(istep, 1, g4gpu.STAGE_PUSH)
            src = oracle.deposit_source(lat, istep, h.get_beam(), cur, LAMBDA0, 1, NG, GRIDMAX)
            h.run(istep, 1, g4gpu.STAGE_FIELD)  # deposition from the same beam + ADI
            want = h.get_field(0)[0]
            before = f_dev.cpu().numpy().astype(np.complex128)
            s_dev = to_device(torch, src)
            delz, dgrid, xks = step_args(lat, istep)
            g4gpu.adi_advance_noalloc(f_dev.data_ptr(), s_dev.data_ptr(), NS, NG, first, delz, dgrid, xks)
            got = f_dev.cpu().numpy().astype(np.complex128)
            assert close(got, want), (istep, np.max(np.abs(got - want)), np.max(np.abs(want)))
            # the source moves the field by far more than the tolerance
            free = oracle.adi_advance(before, None, first, delz, dgrid, xks)
            assert np.max(np.abs(free - want)) > 100 * TOL * np.max(np.abs(want))


def test_noalloc_matches_handle_step_without_source(lib):
    import torch
    import g4gpu
    first = 0
    h, lat, _ = setup_window(first)
    iq = int(np.nonzero(lat[:, 0] == 0)[0][0])  # the quadrupole: no deposition
    with h:
        f_dev = to_device(torch, h.get_field(0)[0])
        for _ in range(2):
            h.run(iq, 1, g4gpu.STAGE_FIELD)
            want = h.get_field(0)[0]
            delz, dgrid, xks = step_args(lat, iq)
            g4gpu.adi_advance_noalloc(f_dev.data_ptr(), None, NS, NG, first, delz, dgrid, xks)
            got = f_dev.cpu().numpy().astype(np.complex128)
            assert close(got, want), (np.max(np.abs(got - want)), np.max(np.abs(want)))


@pytest.mark.parametrize("ns,ng,first", [(401, 51, 100), (300, 168, 7)])
def test_noalloc_window_larger_than_the_grid_matches_oracle(lib, oracle, ns, ng, first):
    import torch
    import g4gpu
    rng = np.random.default_rng(ns)
    shape = (ns, ng * ng)
    field = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    src = 0.1 * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape))
    field = field.astype(np.complex64).astype(np.complex128)
    src = src.astype(np.complex64).astype(np.complex128)
    delz, dgrid, xks = 0.015, 2 * GRIDMAX / (ng - 1), 4.0 * math.asin(1) / LAMBDA0
    f_dev, s_dev = to_device(torch, field), to_device(torch, src)
    want = field
    for _ in range(2):
        want = oracle.adi_advance(want, src, first, delz, dgrid, xks)
        g4gpu.adi_advance_noalloc(f_dev.data_ptr(), s_dev.data_ptr(), ns, ng, first, delz, dgrid, xks)
        got = f_dev.cpu().numpy().astype(np.complex128)
        assert close(got, want), (np.max(np.abs(got - want)), np.max(np.abs(want)))


def test_noalloc_rejects_sizes_beyond_its_limits(lib):
    import torch
    import g4gpu
    buf = torch.zeros(2 * 4 * 169 * 169 + 8, dtype=torch.float32, device="cuda")
    p = buf.data_ptr()
    args = (0.015, 2e-6, 6e10)
    with pytest.raises(g4gpu.G4Error) as e:
        g4gpu.adi_advance_noalloc(p, None, 4, g4gpu.NOALLOC_MAX_NGRID + 1, 0, *args)
    assert e.value.code == g4gpu.ERR_ARG and str(g4gpu.NOALLOC_MAX_NGRID) in str(e.value)
    bad = [((p, None, 0, 51, 0), "nslice"), ((p, None, 4, 2, 0), "ngrid"), ((p, None, 4, 51, 4), "first"),
           ((p + 4, None, 4, 51, 0), "aligned"), ((p, p + 8, 4, 51, 0), "overlaps"), ((0, None, 4, 51, 0), "null")]
    for a, word in bad:
        with pytest.raises(g4gpu.G4Error) as e:
            g4gpu.adi_advance_noalloc(*a, *args)
        assert e.value.code == g4gpu.ERR_ARG and word in str(e.value), (a, str(e.value))
    torch.cuda.synchronize()
