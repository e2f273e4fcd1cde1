"""CPU checks of the C ABI library: it loads without a GPU, exports every symbol
that include/g4gpu.h declares, rejects bad configurations, and its host-side
loading (quiet loading, shot noise, Gauss-Hermite seed, coupling fc) and the
single-particle wakes are bit-exact with the reference's fixtures."""
import os
import platform
import re

import numpy as np
import pytest

from conftest import ROOT, golden

EXACT = platform.machine() in ("x86_64", "AMD64")


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "g4gpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(g4gpu_[a-z_0-9]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(lib):
    import g4gpu
    syms = header_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), s
    assert sorted(g4gpu.ABI_SYMBOLS) == syms


def test_config_defaults_follow_the_reference(lib):
    import g4gpu
    c = g4gpu.Config()
    assert c.npart == 8192 and c.ngrid == 151 and c.nfield == 1 and c.harm[0] == 1
    assert c.lambda0 == 1e-10 and abs(c.gammaref - 5800 / 0.511) < 1e-9
    assert c.xcut == 1 and c.ycut == 1 and c.sigmoid == 1


@pytest.mark.parametrize("bad", [dict(nslice=0), dict(npart=0), dict(ngrid=2), dict(precision=7),
                                 dict(solver=5), dict(gammaref=0.5), dict(sample=0.0)])
def test_create_rejects_bad_configs(lib, bad):
    import g4gpu
    kw = dict(nslice=2, npart=8, ngrid=11, gridmax=1e-4)
    kw.update(bad)
    with pytest.raises(g4gpu.G4Error) as e:
        g4gpu.Handle(g4gpu.Config(**kw))
    assert e.value.code == 1  # G4GPU_ERR_ARG, decided before any device is touched


@pytest.mark.parametrize("name", ["quiet_nb4", "shot_nb4", "shot_nb8", "bunch_emod", "shot_profile"])
def test_host_loading_matches_reference(lib, name):
    import g4gpu
    d = golden("loading.npz")
    islice0, npart, nbins, seed, sn = (int(v) for v in d[name + "_args"])
    got = g4gpu.host_load_beam(d[name + "_sp"], islice0, npart, nbins, seed, sn, 1e-10, 1.0)
    if EXACT:
        assert np.array_equal(got, d[name])
    else:
        assert np.allclose(got, d[name], rtol=1e-14, atol=0)


def test_host_loading_rejects_npart_not_multiple_of_nbins(lib):
    import g4gpu
    d = golden("loading.npz")
    with pytest.raises(g4gpu.G4Error):
        g4gpu.host_load_beam(d["quiet_nb4_sp"], 0, 30, 4, 1, 0, 1e-10, 1.0)


@pytest.mark.parametrize("name", ["gh_fund", "gh_h3"])
def test_host_gauss_hermite_matches_reference(lib, name):
    import g4gpu
    d = golden("loading.npz")
    gm, ng = d[name + "_grid"]
    got = g4gpu.host_gauss_hermite(d[name + "_par"], gm, int(ng))
    assert np.array_equal(got, d[name]) if EXACT else np.allclose(got, d[name], rtol=1e-14)


@pytest.mark.parametrize("name", ["cu_round", "al_flat", "geo_round", "geo_flat", "rough", "all"])
def test_host_single_wakes_match_reference(lib, name):
    """Resistive wall (round pipe, flat chamber), geometric and roughness wakes of the
    &wake settings of tests/golden/wakes.npz against the reference's Wake class."""
    import g4gpu
    d = golden("wakes.npz")
    ns, ds = d["single_ns_ds"]
    radius, cond, relax, roundpipe, gap, lgap, hrough, lrough = d[f"single_{name}_par"]
    got = g4gpu.host_single_wakes(int(ns), ds, radius=radius, conductivity=cond, relaxation=relax,
                                  roundpipe=bool(roundpipe), gap=gap, lgap=lgap, hrough=hrough, lrough=lrough)
    for k, g in zip(("res", "geo", "rou"), got):
        want = d[f"single_{name}_{k}"]
        if EXACT:
            assert np.array_equal(g, want), k
        else:
            assert np.allclose(g, want, rtol=1e-12, atol=1e-12 * np.abs(want).max()), k


def test_host_single_wakes_reject_bad_arguments(lib):
    import g4gpu
    for kw in (dict(ns=0, ds=1e-10), dict(ns=8, ds=0.0), dict(ns=8, ds=1e-10, radius=0.0),
               dict(ns=8, ds=1e-10, gap=1e-3, lgap=0.0), dict(ns=8, ds=1e-10, hrough=1e-7, lrough=0.0)):
        with pytest.raises(g4gpu.G4Error):
            g4gpu.host_single_wakes(**kw)


def test_host_fc_matches_reference(lib):
    import g4gpu
    d = golden("streams.npz")
    fc = np.array([[[g4gpu.host_fc(a, hel, h) for h in range(1, 8)] for hel in (0, 1)] for a in d["fc_aw"]])
    assert np.array_equal(fc, d["fc"]) if EXACT else np.allclose(fc, d["fc"], rtol=1e-14)


def test_large_shot_noise_window_is_sequential_in_slice_order(lib, oracle):
    """The shot-noise stream runs over slices in order even though the quiet loading
    is spread over threads: loading slices 0..N-1 at once equals the oracle."""
    import g4gpu
    import g4cases as T
    sp = T.slice_params(37, 11357.8, 2.0, 0.4e-6, 15.0)
    a = g4gpu.host_load_beam(sp, 0, 32, 4, 7, 1, 1e-10, 1.0)
    b = oracle.load_beam(sp, 0, 32, 4, 7, 1, 1e-10, 1.0)
    assert np.array_equal(a, b)


def test_window_values_rebuilt_from_slices_match_reference_sums(lib, oracle):
    """g4gpu_diag_global (host only) rebuilds the window ("Global/") values from the
    per-slice diagnostics; the oracle forms them from the raw sums over particles and
    cells as DiagBeam / DiagField do (Diagnostic.cpp:551-606, 902-975). Uneven
    currents, a window whose slices differ in power, two fields at harmonics 1 and 3."""
    import g4gpu
    import g4cases as T
    ns, npart, ng = 5, 64, 21
    gms, lam, sample = [6e-5, 4e-5], 1e-10, 1.0
    part = oracle.load_beam(T.slice_params(ns, 11357.8, 2.0, 0.4e-6, 15.0), 0, npart, 4, 3, 1, lam, sample)
    part[..., 2] += np.linspace(0, 3e-6, ns)[:, None]  # slices with different centroids
    cur = np.array([500.0, 3000.0, 2500.0, 1200.0, 3000.0])
    x = np.arange(ng) - 0.5 * (ng - 1)
    g = np.exp(-((x[None, :] - 1.0) ** 2 + (x[:, None] + 0.5) ** 2) / (0.05 * ng * ng))
    fld = np.stack([np.stack([(g * (1 + s) * np.exp(1j * (0.1 * s + 0.05 * k) * x[None, :])).ravel() * 1e4
                              for s in range(ns)]) for k in range(2)])
    first = 2
    cfg = g4gpu.Config(nslice=ns, npart=npart, ngrid=ng, harm=[1, 3], gridmax=gms, lambda0=lam, sample=sample,
                       gammaref=11357.8)
    bd = oracle.diag_beam(part, 1)
    fd = np.stack([oracle.diag_field(fld[k], gms[k], lam, h, first) for k, h in enumerate([1, 3])])
    qd = np.stack([oracle.diag_field_fft(fld[k], gms[k], lam, h, first) for k, h in enumerate([1, 3])])
    # the per-slice outputs are by window slice; the current too
    cur_w = cur
    bg, fg = g4gpu.diag_global(cfg, 1, cur_w, bd, fd, qd)
    want_b = oracle.diag_global_beam(part, cur_w)
    assert np.allclose(bg, want_b, rtol=1e-9, atol=1e-12 * np.abs(want_b).max())
    for k, h in enumerate([1, 3]):
        want_f = oracle.diag_global_field(fld[k], gms[k], lam, h, sample)
        for col in range(len(want_f)):
            scale = abs(want_f[col]) if col in (0, 5, 6) else np.abs(want_f[[1, 2, 3, 4]]).max() \
                if col <= 4 else np.abs(want_f[7:]).max()
            assert abs(fg[k][col] - want_f[col]) <= 1e-9 * scale, (k, col, fg[k][col], want_f[col])
    # without the far-field input the far-field columns are zero
    _, fg0 = g4gpu.diag_global(cfg, 1, None, None, fd, None)
    assert np.all(fg0[:, 7:] == 0) and np.allclose(fg0[:, :7], fg[:, :7])


def _plugin_field_case(ns=5, ng=13):
    rng = np.random.default_rng(7)
    f = (rng.standard_normal((ns, ng * ng)) + 1j * rng.standard_normal((ns, ng * ng))) * (1 + np.arange(ns))[:, None]
    return f


@pytest.mark.parametrize("kind", ["field", "multi"])
def test_plugin_runner_feeds_slices_by_window_order(lib, test_plugins, kind):
    """The plugin runner (DiagFieldHook's feeding, DiagnosticHook.cpp:110-262) on a
    test plugin built against include/g4gpu_dpi_abi.h: slice by slice in storage order
    or all at once, each value stored at its window slice (is = (ns + is0 - first) % ns)."""
    import g4gpu
    ns, ng, first = 5, 13, 3
    f = _plugin_field_case(ns, ng)
    with g4gpu.Plugin(test_plugins[kind]) as p:
        assert p.kind == g4gpu.G4GPU_DPI_FIELD and p.multi == (kind == "multi")
        assert p.names == ["sum_abs2", "slice", "iz"] and p.info == "test field plugin"
        out = p.field(f, first, iz=7, harm=1, ngrid=ng, dgrid=1e-6, xlambda=1e-10)
    for is0 in range(ns):
        is_ = (ns + is0 - first) % ns
        assert out["sum_abs2"][is_] == pytest.approx(np.sum(np.abs(f[is0]) ** 2), rel=1e-14)
    assert np.array_equal(out["slice"], np.arange(ns)) and np.all(out["iz"] == 7)


def test_plugin_runner_beam(lib, test_plugins):
    import g4gpu
    rng = np.random.default_rng(3)
    part = rng.standard_normal((4, 16, 6)) + 100.0
    with g4gpu.Plugin(test_plugins["beam"]) as p:
        assert p.kind == g4gpu.G4GPU_DPI_BEAM and p.names == ["mean_gamma", "slice"]
        out = p.beam(part, iz=0)
    assert np.allclose(out["mean_gamma"], part[..., 0].mean(axis=1), rtol=1e-14)
    assert np.array_equal(out["slice"], np.arange(4))


def test_plugin_runner_rejects_non_plugins(lib, tmp_path):
    import g4gpu
    with pytest.raises(g4gpu.G4Error):
        g4gpu.Plugin(str(tmp_path / "missing.so"))
    with pytest.raises(g4gpu.G4Error, match="factory"):
        g4gpu.Plugin(g4gpu.LIB_PATH)  # a library that is no plugin


def test_reference_demo_plugins_run_in_the_engine(lib):
    """The reference's own demo plugins (misc/plugin_demo, built unmodified from their
    sources into oracle/_ref by oracle/ref_build): the field demo's power agrees with the
    core's power formula (with the demo's constant eev = 510999.06), the beam demo's
    x standard deviation with numpy."""
    import g4gpu
    here = os.path.dirname(os.path.abspath(__file__))
    ref = os.path.join(os.path.dirname(here), "oracle", "_ref")
    fdemo, bdemo = os.path.join(ref, "libdemo.so"), os.path.join(ref, "libbeamdemo.so")
    if not (os.path.exists(fdemo) and os.path.exists(bdemo)):
        pytest.skip("the reference's demo plugins are not built here")
    ns, ng, first, gm, lam = 5, 13, 2, 5e-5, 1e-10
    f = _plugin_field_case(ns, ng)
    dgrid = 2 * gm / (ng - 1)
    try:
        p = g4gpu.Plugin(fdemo)
    except g4gpu.G4Error as e:  # built for another machine
        pytest.skip(str(e))
    with p:
        assert p.names == ["my_power", "abc"]
        out = p.field(f, first, iz=0, harm=1, ngrid=ng, dgrid=dgrid, xlambda=lam)
    ks = 4 * np.arcsin(1.0) / lam
    scl = dgrid * 510999.06 / ks
    for is0 in range(ns):
        want = np.sum(np.abs(f[is0]) ** 2) * scl * scl / 376.73
        assert out["my_power"][(ns + is0 - first) % ns] == pytest.approx(want, rel=1e-13)
    assert np.all(out["abc"] == 42.0)
    rng = np.random.default_rng(5)
    part = rng.standard_normal((3, 32, 6))
    with g4gpu.Plugin(bdemo) as p:
        assert p.names == ["xstd", "the_answer"]
        out = p.beam(part, iz=0)
    assert np.allclose(out["xstd"], part[..., 2].std(axis=1), rtol=1e-13)
    assert np.all(out["the_answer"] == 42.0)


def test_h5_writer_round_trip(lib, tmp_path):
    """The HDF5 encoder against a reader written from the file format specification
    (tests/h5read.py): nested groups, groups of more than one symbol table node (8
    entries), 1-D and 2-D datasets, an empty one, the unit attributes."""
    import g4gpu
    import h5read
    rng = np.random.default_rng(0)
    path = str(tmp_path / "x.h5")
    want = {}
    with g4gpu.H5Writer(path) as w:
        for i in range(40):
            a = rng.normal(size=(3, 5))
            w.dataset(f"Beam/d{i:02d}", a, "m")
            want[f"d{i:02d}"] = a
        w.dataset("Lattice/aw", np.arange(7.0), " ")
        w.dataset("Field3/Global/energy", np.arange(3.0), "J")
        w.dataset("Meta/empty", np.zeros((0, 4)), "x")
    t = h5read.read(path)
    assert sorted(t) == ["Beam", "Field3", "Lattice", "Meta"]
    for k, a in want.items():
        d, attrs = t["Beam"][k]
        assert np.array_equal(d, a) and attrs == {"unit": "m"}
    assert np.array_equal(t["Lattice"]["aw"][0], np.arange(7.0)) and t["Lattice"]["aw"][1]["unit"] == " "
    assert np.array_equal(t["Field3"]["Global"]["energy"][0], np.arange(3.0))
    assert t["Meta"]["empty"][0].shape == (0, 4)
    # lookups by name through the B-tree keys, as the HDF5 library finds members
    for k, a in want.items():
        assert np.array_equal(h5read.get(path, f"Beam/{k}")[0], a)
    with pytest.raises(KeyError):
        h5read.get(path, "Beam/nothing")


def test_h5_writer_groups_of_thousands(lib, tmp_path):
    """A dump of 3000 slices: the root group's B-tree takes an internal level above its
    leaves; every slice is found by name; integer datasets."""
    import g4gpu
    import h5read
    import outfile
    ns, ng = 3000, 5
    cfg = g4gpu.Config(nslice=ns, npart=8, ngrid=ng, gridmax=1e-4, lambda0=1e-10, sample=1.0, gammaref=1e4)
    rng = np.random.default_rng(0)
    fld = rng.normal(size=(ns, ng * ng)) + 1j * rng.normal(size=(ns, ng * ng))
    path = str(tmp_path / "a.fld.h5")
    outfile.write_fld(path, cfg, 0, fld, 7)
    t = h5read.read(path)
    assert len(t) == ns + 7 and t["gridpoints"][0].tolist() == [ng] and t["slicecount"][0].tolist() == [ns]
    scl = (2e-4 / (ng - 1)) * 510998.95069 / (2 * np.pi / 1e-10) / np.sqrt(376.73)
    for i in (0, 1, 777, 2999):
        got = h5read.get(path, f"slice{i + 1:06d}/field-imag")[0]
        assert np.allclose(got, scl * fld[(i + 7) % ns].imag, rtol=1e-15)
    part = rng.normal(size=(4, 8, 6))
    path = str(tmp_path / "a.par.h5")
    cfg4 = g4gpu.Config(nslice=4, npart=8, ngrid=ng, gridmax=1e-4, lambda0=1e-10, sample=1.0, gammaref=1e4)
    outfile.write_par(path, cfg4, part, np.arange(4.0), 4, counts=[8, 5, 0, 3])
    assert h5read.get(path, "one4one")[0].tolist() == [1]
    assert np.array_equal(h5read.get(path, "slice000002/theta")[0], part[1, :5, 1])
    assert h5read.get(path, "slice000003/x")[0].shape == (0,)


def test_h5_writer_rejects_duplicates_and_bad_paths(lib, tmp_path):
    import g4gpu
    w = g4gpu.H5Writer(str(tmp_path / "y.h5"))
    w.dataset("A/b", [1.0], "m")
    with pytest.raises(g4gpu.G4Error):
        w.dataset("A/b", [2.0], "m")
    with pytest.raises(g4gpu.G4Error):
        w.dataset("A/b/c", [2.0], "m")  # b is a dataset
    w.close()
