"""The reference's output file (.out.h5 layout) from a run's device diagnostics, written by
the engine's HDF5 encoder and read back with the specification reader tests/h5read.py."""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [0, 1])
def test_out_file_holds_the_run_diagnostics(lib, tmp_path, prec):
    import g4gpu
    import h5read
    import outfile
    d = golden("steps.npz")
    g = lambda k: d[f"harm13_{k}"]
    gammaref, time_run, periodic = g("args")
    part, fields = g("part"), g("fields")
    ns, npart = part.shape[0], part.shape[1]
    ng = int(round(np.sqrt(fields.shape[2])))
    cfg = g4gpu.Config(nslice=ns, npart=npart, ngrid=ng, harm=list(g("harm")), gridmax=list(g("gridmax")),
                       lambda0=1e-10, sample=1.0, gammaref=float(gammaref), precision=prec, time_run=int(time_run),
                       periodic=int(periodic))
    lat = g("lat")
    nh = 3
    with g4gpu.Handle(cfg) as h:
        h.set_lattice(lat)
        h.load_beam(part, g("cur"))
        for k in range(fields.shape[0]):
            h.load_field(k, fields[k], first=int(g("first")[k]))
        beam, field = h.run_diag(0, lat.shape[0], nharm=nh)
    zout = lat[:, 17] + lat[:, 13]
    path = str(tmp_path / "run.out.h5")
    outfile.write_out(path, cfg, lat, zout, beam, field, g("cur"), nharm=nh)
    t = h5read.read(path)
    assert {"Lattice", "Global", "Beam", "Field", "Field3", "Meta"} <= set(t)
    e, a = t["Beam"]["energy"]
    assert np.array_equal(e, beam[:, :, 0]) and a["unit"] == "mc^2"
    assert np.array_equal(t["Beam"]["bunching3"][0], beam[:, :, len(g4gpu.DB_COLS) + 4])
    assert np.array_equal(t["Beam"]["current"][0], np.tile(g("cur"), (lat.shape[0], 1)))
    p, a = t["Field"]["power"]
    assert np.array_equal(p, field[:, 0, :, 0]) and a["unit"] == "W"
    assert np.array_equal(t["Field3"]["xsize"][0], field[:, 1, :, 2])
    assert np.array_equal(t["Lattice"]["aw"][0], lat[:, 0]) and t["Lattice"]["zplot"][0].shape == (lat.shape[0],)
    assert np.allclose(t["Global"]["s"][0], np.arange(ns) * 1e-10)
    # window energy of the last step: the power summed over the slices (times the slice's time)
    fg = g4gpu.diag_global(cfg, nh, g("cur"), None, field[-1], None)[1]
    assert np.isclose(t["Field"]["Global"]["energy"][0][-1], fg[0][0])
