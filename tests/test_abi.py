"""CPU checks of the C ABI library: it loads without a GPU, exports every symbol
that include/g4gpu.h declares, rejects bad configurations, and its host-side
loading (quiet loading, shot noise, Gauss-Hermite seed, coupling fc) is bit-exact
with the reference's fixtures."""
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
