"""The reference-side binding of the engine (GencoreGPU, genesis-1.3-version4_gb300/
integration) compiled against the reference's own, unmodified headers and linked with
the reference's objects and the engine's library (oracle/ref_build/Makefile builds
oracle/_ref/gencore_gpu_check where the reference's source tree is present). The check
program runs a small deck through Gencore::run and GencoreGPU::run: with a GPU the two
must agree within 1e-9; without one, GencoreGPU::run must refuse before any step so
that the caller keeps Gencore::run."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CHECK = os.path.join(ROOT, "oracle", "_ref", "gencore_gpu_check")


def test_gencore_gpu_binding_builds_and_runs(tmp_path):
    if not os.path.exists(CHECK):
        pytest.skip("the reference checker (and with it the binding check) is built only where the "
                    "reference's source tree is present")
    r = subprocess.run([CHECK], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    last = r.stdout.strip().splitlines()[-1]
    assert last.startswith("FALLBACK") or last.startswith("MATCH"), last
