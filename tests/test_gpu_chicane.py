"""Chicanes on the device (TrackBeam::applyChicane before the first half step of the
chicane's step, TrackBeam::applyR56 after its integration), through the C ABI, against
the reference run (tests/golden/chicane.npz, bit-exact with the oracle) and the oracle.

Tolerances as for space charge: plain FP64 1e-9 of the largest change over the run
(gamma, theta) or of the largest value; mixed form 1 % of the chicane's effect on theta
(the run with the chicane minus the run without it), which R56 makes about 2000 rad here.
"""
import numpy as np
import pytest

from conftest import golden
from test_gpu_space_charge import assert_plain_like, rel

pytestmark = pytest.mark.gpu


def fixture(case):
    d = golden("chicane.npz")
    return lambda k: d[f"{case}_{k}"]


def run_fixture(g, precision, chicane=True, efield=None, graph=False):
    import g4gpu
    gammaref, time_run, periodic = g("args")
    part, fields = g("part"), g("fields")
    ns, npart = part.shape[0], part.shape[1]
    ngrid = int(round(np.sqrt(fields.shape[2])))
    cfg = g4gpu.Config(nslice=ns, npart=npart, ngrid=ngrid, harm=list(g("harm")), gridmax=list(g("gridmax")),
                       lambda0=1e-10, sample=1.0, gammaref=float(gammaref), precision=precision,
                       time_run=int(time_run), periodic=int(periodic))
    with g4gpu.Handle(cfg) as h:
        h.set_lattice(g("lat"))
        if chicane:
            h.set_chicanes(g("chic"))
        h.load_beam(part, g("cur"))
        for k in range(fields.shape[0]):
            h.load_field(k, fields[k], first=int(g("first")[k]))
        if efield:
            h.set_efield(*efield)
        h.set_graph_mode(graph)
        h.run(0, g("lat").shape[0])
        return h.get_beam(), [h.get_field(k)[:2] for k in range(fields.shape[0])]


@pytest.mark.parametrize("case,graph", [("td", False), ("steady", False), ("td", True)])
def test_plain_chicane_matches_reference(lib, case, graph):
    g = fixture(case)
    p, f = run_fixture(g, 0, graph=graph)
    assert_plain_like(p, f, g("part"), g("out_part"), g("out_fields"), g("out_first"))
    q, _ = run_fixture(g, 0, chicane=False)
    assert rel(q[..., 2], g("out_part")[..., 2]) > 1e-7  # the chicane's matrix is visible in x


@pytest.mark.parametrize("case", ["td", "steady"])
def test_mixed_chicane_within_one_percent(lib, case):
    g = fixture(case)
    m_c, _ = run_fixture(g, 1)
    m_n, _ = run_fixture(g, 1, chicane=False)
    q_n, _ = run_fixture(g, 0, chicane=False)
    assert rel(m_c[..., 1] - m_n[..., 1], g("out_part")[..., 1] - q_n[..., 1]) < 1e-2


@pytest.mark.parametrize("prec", [0, 1])
def test_chicane_with_space_charge_matches_oracle(lib, oracle, prec):
    """The chicane in the first half step that the space-charge moment kernel runs."""
    g = fixture("td")
    ef = (0.0, 24, 2, 1, True)
    gammaref, time_run, periodic = g("args")
    oracle.set_chicanes(g("chic"))
    oracle.set_efield(*ef)
    try:
        rp, rf, rfirst, _ = oracle.run_steps(g("lat"), gammaref, g("part"), g("cur"), 1e-10, 1.0, g("harm"),
                                             g("gridmax"), g("fields"), g("first"), time_run=int(time_run),
                                             periodic=int(periodic), stages=7)
    finally:
        oracle.set_chicanes()
        oracle.set_efield()
    if prec == 0:
        p, f = run_fixture(g, 0, efield=ef)
        assert_plain_like(p, f, g("part"), rp, rf, rfirst)
    else:
        m, _ = run_fixture(g, 1, efield=ef)
        m_n, _ = run_fixture(g, 1, chicane=False, efield=ef)
        q_n, _ = run_fixture(g, 0, chicane=False, efield=ef)
        assert rel(m[..., 1] - m_n[..., 1], rp[..., 1] - q_n[..., 1]) < 1e-2


def test_set_chicanes_rejects_bad_tables(lib):
    import g4gpu
    g = fixture("td")
    cfg = g4gpu.Config(nslice=4, npart=64, ngrid=25, gridmax=6e-5, lambda0=1e-10, sample=1.0, gammaref=11357.8)
    with g4gpu.Handle(cfg) as h:
        h.set_lattice(g("lat"))
        chic = g("chic")
        with pytest.raises(g4gpu.G4Error):
            h.set_chicanes(chic[:-1])  # one row short
        bad = chic.copy()
        bad[6, 1] = 0.0  # lb 0
        with pytest.raises(g4gpu.G4Error):
            h.set_chicanes(bad)
        h.set_chicanes(chic)
        h.set_chicanes(np.zeros_like(chic))  # none


@pytest.mark.parametrize("slip", [10.3, 3.0, -6.2])
def test_long_slippage_clears_like_the_oracle(lib, oracle, slip):
    """A step whose slippage enters more slices than the window holds (a chicane's
    delay): every slice cleared once and the ring start moved by the full count, as the
    reference's slice-by-slice loop leaves them; also a shorter and a backward one."""
    import g4gpu
    g = fixture("td")
    lat = g("lat").copy()
    lat[6, 14] = slip  # the chicane row's slippage (column "slip")
    gammaref, time_run, periodic = g("args")
    oracle.set_chicanes(g("chic"))
    try:
        rp, rf, rfirst, _ = oracle.run_steps(lat, gammaref, g("part"), g("cur"), 1e-10, 1.0, g("harm"), g("gridmax"),
                                             g("fields"), g("first"), time_run=1, periodic=0, stages=7)
    finally:
        oracle.set_chicanes()
    part, fields = g("part"), g("fields")
    cfg = g4gpu.Config(nslice=4, npart=part.shape[1], ngrid=25, gridmax=6e-5, lambda0=1e-10, sample=1.0,
                       gammaref=float(gammaref), time_run=1)
    with g4gpu.Handle(cfg) as h:
        h.set_lattice(lat)
        h.set_chicanes(g("chic"))
        h.load_beam(part, g("cur"))
        h.load_field(0, fields[0], first=int(g("first")[0]))
        h.run(0, lat.shape[0])
        p = h.get_beam()
        f, first, _ = h.get_field(0)
    assert_plain_like(p, [(f, first)], part, rp, rf, rfirst)
