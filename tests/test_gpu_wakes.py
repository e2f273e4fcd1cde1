"""Wakes (&wake) on the device, through the C ABI, against the reference run with its
own Collective (tests/golden/wakes.npz, bit-exact with the oracle:
tests/test_oracle_pins.py) and against the oracle for cases made here.

Tolerances as for space charge: plain FP64 1e-9 of the largest change over the run
(gamma, theta) or of the largest value (x, y, px, py, fields) — the device sums each
slice's wake in another order than the reference's loop; mixed form 1 % of the largest
wake effect on gamma.
"""
import numpy as np
import pytest

from conftest import golden
from test_gpu_space_charge import assert_plain_like, made_case, rel

pytestmark = pytest.mark.gpu

CASES = ["s1", "s1_transient", "s3"]


def fixture(case):
    d = golden("wakes.npz")
    return lambda k: d[f"{case}_{k}"]


def run_fixture(g, precision, wake=True, graph=False, wake_before_beam=False, efield=None):
    import g4gpu
    gammaref, time_run, periodic, sample = g("args")
    part, fields = g("part"), g("fields")
    ns, npart = part.shape[0], part.shape[1]
    ngrid = int(round(np.sqrt(fields.shape[2])))
    cfg = g4gpu.Config(nslice=ns, npart=npart, ngrid=ngrid, harm=list(g("harm")), gridmax=list(g("gridmax")),
                       lambda0=1e-10, sample=float(sample), gammaref=float(gammaref), precision=precision,
                       time_run=int(time_run), periodic=int(periodic))
    lat = g("lat")
    ds, ztrans, radius, transient = g("wake_par")
    with g4gpu.Handle(cfg) as h:
        h.set_lattice(lat)
        setw = lambda: h.set_wake(g("wake_ext"), g("wake_res"), g("wake_geo"), g("wake_rou"), ds, ztrans, radius,
                                  bool(transient))
        if wake and wake_before_beam:
            setw()
        h.load_beam(part, g("cur"))
        for k in range(fields.shape[0]):
            h.load_field(k, fields[k], first=int(g("first")[k]))
        if wake and not wake_before_beam:
            setw()
        if efield:
            h.set_efield(*efield)
        h.set_graph_mode(graph)
        h.run(0, lat.shape[0])
        return h.get_beam(), [h.get_field(k)[:2] for k in range(fields.shape[0])]


@pytest.mark.parametrize("case", CASES)
def test_plain_wakes_match_reference(lib, case):
    g = fixture(case)
    p, f = run_fixture(g, 0)
    assert_plain_like(p, f, g("part"), g("out_part"), g("out_fields"), g("out_first"))
    q, _ = run_fixture(g, 0, wake=False)
    p0 = g("part")[..., 0]
    assert rel(q[..., 0] - p0, g("out_part")[..., 0] - p0) > 1e-6  # the wake is visible


@pytest.mark.parametrize("graph,before", [(True, False), (False, True)])
def test_plain_wakes_in_graphs_and_set_before_the_beam(lib, graph, before):
    """Captured step graphs, and a wake set before the beam is loaded (its slices'
    wake is then formed from the current the load brings)."""
    g = fixture("s3")
    p, f = run_fixture(g, 0, graph=graph, wake_before_beam=before)
    assert_plain_like(p, f, g("part"), g("out_part"), g("out_fields"), g("out_first"))


@pytest.mark.parametrize("case", CASES)
def test_mixed_wakes_within_one_percent(lib, case):
    g = fixture(case)
    m_w, _ = run_fixture(g, 1)
    m_n, _ = run_fixture(g, 1, wake=False)
    q_n, _ = run_fixture(g, 0, wake=False)
    assert rel(m_w[..., 0] - m_n[..., 0], g("out_part")[..., 0] - q_n[..., 0]) < 1e-2, case


@pytest.mark.parametrize("prec", [0, 1])
def test_wakes_with_space_charge_match_oracle(lib, oracle, prec):
    """Wakes and space charge in one step (the wake after the integration, before the
    second transverse half step), on a made window: plain against the oracle at 1e-9,
    mixed within 1 % of the combined effect."""
    import g4gpu
    gref, ng, gm, lat, part, cur, fld = case = made_case(ns=6, npart=128)
    ns = part.shape[0]
    res, geo, rou = g4gpu.host_single_wakes(ns, 1e-10, radius=2e-3, conductivity=5.813e7, relaxation=8.1e-6,
                                            gap=1e-3, lgap=0.5, hrough=1e-7, lrough=1e-4)
    res, geo, rou = res * 1e2, geo * 30.0, rou * 1e3
    ext = np.linspace(-800.0, 800.0, ns)
    ef = (0.0, 40, 2, 1, True)

    def engine(precision, on):
        cfg = g4gpu.Config(nslice=ns, npart=part.shape[1], ngrid=ng, gridmax=gm, lambda0=1e-10, sample=1.0,
                           gammaref=gref, precision=precision, time_run=1)
        with g4gpu.Handle(cfg) as h:
            h.set_lattice(lat)
            h.load_beam(part, cur)
            h.load_field(0, fld)
            if on:
                h.set_wake(ext, res, geo, rou)
                h.set_efield(*ef)
            h.run(0, lat.shape[0])
            return h.get_beam(), h.get_field(0)[:2]

    oracle.set_wake(ext, res, geo, rou, 1e-10)
    oracle.set_efield(*ef)
    try:
        rp, rf, rfirst, _ = oracle.run_steps(lat, gref, part, cur, 1e-10, 1.0, [1], [gm], fld[None], [0])
    finally:
        oracle.set_wake()
        oracle.set_efield()
    if prec == 0:
        p, (f, first) = engine(0, True)
        assert_plain_like(p, [(f, first)], part, rp, rf, rfirst)
    else:
        q_no, _ = engine(0, False)
        m_on, _ = engine(1, True)
        m_no, _ = engine(1, False)
        assert rel(m_on[..., 0] - m_no[..., 0], rp[..., 0] - q_no[..., 0]) < 1e-2


def test_set_wake_rejects_bad_arguments(lib):
    import g4gpu
    cfg = g4gpu.Config(nslice=4, npart=64, ngrid=21, gridmax=1e-4, lambda0=1e-10, sample=1.0, gammaref=11357.8)
    z4, z2 = np.zeros(4), np.zeros(2)
    with g4gpu.Handle(cfg) as h:
        with pytest.raises(g4gpu.G4Error):
            h.set_wake(z4, z2, z2, z2)  # fewer fine points than slices
        with pytest.raises(g4gpu.G4Error):
            h.set_wake(z4, z4, z4, z4, ds=0.0)
        h.set_wake(z4, z4, z4, z4)
        h.set_wake()  # off
