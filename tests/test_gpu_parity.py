"""GPU parity tests: the CUDA path, called through the C ABI, against the reference.

References used:
  * tests/golden/steps.npz, example1.npz, config0.npz — produced by the GENESIS 1.3 v4
    reference itself (tests/golden/gen_golden.py);
  * the C restatement oracle/g4oracle.c, bit-exact with those fixtures
    (tests/test_oracle_pins.py), for cases generated on the fly.

Tolerances (relative to the largest magnitude of the compared quantity):
  * plain FP64 path, small windows: 1e-9 — the kernels round every operation as
    the reference does except CUDA's sin/cos/sinh/cosh, which differ in the last bit;
  * plain FP64 path, full decks (Example1: 1104 lasing steps): 1e-6 on the power of
    every step — last-bit differences grow through the FEL gain;
  * mixed form against the plain path: 1 % on slice power and bunching (the target
    of the mixed form).
"""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


def rel_err(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    scale = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / scale) if scale > 0 else float(np.max(np.abs(a - b)))


def handle_for(g4gpu, ns, npart, ngrid, harm, gridmax, gammaref, precision, time_run, periodic):
    cfg = g4gpu.Config(nslice=ns, npart=npart, ngrid=ngrid, harm=list(harm), gridmax=list(gridmax),
                       lambda0=1e-10, sample=1.0, gammaref=float(gammaref), precision=precision,
                       time_run=int(time_run), periodic=int(periodic))
    return g4gpu.Handle(cfg)


def load_case(lib, case, precision, stages):
    import g4gpu
    d = golden("steps.npz")
    g = lambda k: d[f"{case}_{k}"]
    gammaref, time_run, periodic = g("args")
    part, fields = g("part"), g("fields")
    ns, npart = part.shape[0], part.shape[1]
    ngrid = int(round(np.sqrt(fields.shape[2])))
    h = handle_for(g4gpu, ns, npart, ngrid, g("harm"), g("gridmax"), gammaref, precision, time_run, periodic)
    lat = g("lat")[:1] if stages != 7 else g("lat")
    h.set_lattice(lat)
    h.load_beam(part, g("cur"))
    for k in range(fields.shape[0]):
        h.load_field(k, fields[k], first=int(g("first")[k]))
    return h, g, lat.shape[0]


@pytest.mark.parametrize("case", ["planar", "helical", "harm13", "steady"])
@pytest.mark.parametrize("stages", [1, 2, 4, 7])
def test_plain_steps_match_reference(lib, case, stages):
    h, g, nsteps = load_case(lib, case, 0, stages)
    with h:
        h.run(0, nsteps, stages)
        part = h.get_beam()
        ref_p = g(f"s{stages}_part")
        for col in range(6):
            assert rel_err(part[..., col], ref_p[..., col]) < 1e-9, (case, stages, col)
        ref_f = g(f"s{stages}_fields")
        for k in range(ref_f.shape[0]):
            f, first, _ = h.get_field(k)
            assert rel_err(f, ref_f[k]) < 1e-9, (case, stages, k)
            assert first == int(g(f"s{stages}_first")[k])


@pytest.mark.parametrize("case", ["planar", "helical", "harm13", "steady"])
def test_mixed_steps_close_to_reference(lib, oracle, case):
    """Mixed form over whole small lattices: slice power and bunching within 1 %."""
    h, g, nsteps = load_case(lib, case, 1, 7)
    with h:
        h.run(0, nsteps)
        bd, fd = h.diag(nharm=1)
    ref_p = g("s7_part")
    ref_f = g("s7_fields")
    ob = oracle.diag_beam(ref_p, 1)
    assert rel_err(bd[:, 24], ob[:, 24]) < 1e-2, case
    for k in range(ref_f.shape[0]):
        of = oracle.diag_field(ref_f[k], float(g("gridmax")[k]), 1e-10, int(g("harm")[k]),
                               int(g("s7_first")[k]))
        assert rel_err(fd[k][:, 0], of[:, 0]) < 1e-2, (case, k)


def test_beam_and_field_round_trip(lib):
    import g4gpu
    d = golden("steps.npz")
    part, fld = d["harm13_part"], d["harm13_fields"]
    for prec in (0, 1):
        with handle_for(g4gpu, part.shape[0], part.shape[1], 19, [1, 3], [6e-5, 4e-5], 11357.8, prec, 1, 0) as h:
            h.load_beam(part, d["harm13_cur"])
            h.load_field(1, fld[1], first=3, accuslip=0.25)
            h.load_field(0, fld[0], first=0)
            p2 = h.get_beam()
            f2, first, acc = h.get_field(1)
            assert first == 3 and acc == 0.25
            if prec == 0:
                assert np.array_equal(p2, part) and np.array_equal(f2, fld[1])
            else:
                assert np.array_equal(p2[..., 1], part[..., 1])  # theta stays FP64
                assert rel_err(p2, part) < 1e-6 and rel_err(f2, fld[1]) < 1e-6


def test_diagnostics_match_oracle(lib, oracle):
    import g4gpu
    d = golden("steps.npz")
    part, fld = d["planar_s7_part"], d["planar_s7_fields"]
    first = int(d["planar_s7_first"][0])
    with handle_for(g4gpu, 4, 64, 25, [1], [6e-5], 11357.8, 0, 1, 0) as h:
        h.load_beam(part, d["planar_cur"])
        h.load_field(0, fld[0], first=first)
        bd, fd = h.diag(nharm=3)
    ob = oracle.diag_beam(part, 3)
    of = oracle.diag_field(fld[0], 6e-5, 1e-10, 1, first)
    for col in range(ob.shape[1]):
        assert np.allclose(bd[:, col], ob[:, col], rtol=1e-10, atol=1e-14 * np.max(np.abs(ob[:, col])) + 1e-300), col
    for col in range(of.shape[1]):
        assert np.allclose(fd[0][:, col], of[:, col], rtol=1e-10, atol=1e-12 * np.max(np.abs(of[:, col]))), col


def run_deck_fixture(lib, name, precision, every=1):
    import g4gpu
    d = golden(name)
    ng = int(d["ngrid"])
    gm = float(d["gridmax"])
    par = np.array([d["lambda0"], d["power0"], 0, 0, d["waist"], 0, 0, 0, 0, 0, 0, 1.0])
    fld = g4gpu.host_gauss_hermite(par, gm, ng)
    beam = d["beam"]
    with handle_for(g4gpu, 1, beam.shape[1], ng, [1], [gm], float(d["gammaref"]), precision, 0, 0) as h:
        h.set_lattice(d["lat"])
        h.load_beam(beam, d["current"])
        h.load_field(0, fld[None])
        power = [h.diag(1)[1][0, 0, 0]]
        bunch = [h.diag(1)[0][0, 24]]
        n = d["lat"].shape[0]
        for i in range(n):
            h.run(i, 1)
            if (i + 1) % every == 0 or i == n - 1:
                bd, fd = h.diag(1)
                power.append(fd[0, 0, 0])
                bunch.append(bd[0, 24])
    return np.array(power), np.array(bunch), d


def test_example1_plain_matches_reference_every_step(lib):
    power, bunch, d = run_deck_fixture(lib, "example1.npz", 0)
    assert power.shape == d["power"].shape
    err = np.abs(power / d["power"] - 1)
    assert err.max() < 1e-6, err.max()
    assert np.max(np.abs(bunch - d["bunching"])) < 1e-6
    assert abs(power[-1] / 0.932785e9 - 1) < 0.3  # the reference's CI check


def test_example1_mixed_within_one_percent(lib):
    power, bunch, d = run_deck_fixture(lib, "example1.npz", 1, every=8)
    assert abs(power[-1] / d["power"][-1] - 1) < 1e-2
    assert abs(bunch[-1] - d["bunching"][-1]) < 1e-2 * max(d["bunching"][-1], 1e-3)


def test_config0_plain_matches_reference(lib):
    power, bunch, d = run_deck_fixture(lib, "config0.npz", 0)
    assert np.max(np.abs(power / d["power"] - 1)) < 1e-9
    assert np.max(np.abs(bunch - d["bunching"])) < 1e-9


def test_time_dependent_sase_window_matches_oracle(lib, oracle):
    """Shot-noise SASE window (the 4096-slice workload's physics at a size the
    oracle finishes quickly): 48 slices, 512 particles, ngrid 41, one module."""
    import g4gpu
    import g4cases as T
    ns, npart, ng, gm = 48, 512, 41, 1e-4
    cur = T.flat_top_current(ns, 1e-10, 1.0, 3000.0, 0.6e-9)
    lat = T.undulator_lattice(1.7, 0.015, 110, 1, 1e-10, 11357.8)
    beam = g4gpu.host_load_beam(T.slice_params(ns, 11357.8, 2.0, 0.4e-6, 15.0, currents=cur), 0, npart, 4, 7,
                                1, 1e-10, 1.0)
    fld = np.zeros((ns, ng * ng), dtype=np.complex128)
    with handle_for(g4gpu, ns, npart, ng, [1], [gm], 11357.8, 0, 1, 0) as h:
        h.set_lattice(lat)
        h.load_beam(beam, cur)
        h.load_field(0, fld)
        h.run(0, lat.shape[0])
        bd, fd = h.diag(1)
        first = h.slippage_state(0)[0]
    p, f, ofirst, _ = oracle.run_steps(lat, 11357.8, beam, cur, 1e-10, 1.0, [1], [gm], fld[None], [0],
                                       time_run=1, nthreads=8)
    assert first == ofirst[0]
    ob = oracle.diag_beam(p, 1)
    of = oracle.diag_field(f[0], gm, 1e-10, 1, int(ofirst[0]))
    assert rel_err(fd[0][:, 0], of[:, 0]) < 1e-7
    assert rel_err(bd[:, 24], ob[:, 24]) < 1e-7


def test_run_before_load_is_an_error(lib):
    import g4gpu
    with handle_for(g4gpu, 2, 8, 11, [1], [1e-4], 11357.8, 0, 1, 0) as h:
        h.set_lattice(np.zeros((1, g4gpu.LAT_NCOL)))
        with pytest.raises(g4gpu.G4Error) as e:
            h.run(0, 1)
        assert e.value.code == 3
        with pytest.raises(g4gpu.G4Error) as e:
            h.run(0, 5)
        assert e.value.code == 1
