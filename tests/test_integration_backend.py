"""The reference-side GPU back-end (svfsiplus_gb300/integration/GpuLinearAlgebra.{h,cpp},
the LinearAlgebra subclass a reference build selects for this library): compiled
against the reference's own headers (LinearAlgebra.h:40-63, FsilsLinearAlgebra's
includes) and linked with the reference's objects and libsvgpu.so by
oracle/build_ref.sh.  Runs where the reference
tree exists (skipped elsewhere); the linked executable is run without arguments, which
reports the link and touches no GPU."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_gpu_backend_builds_against_reference_headers():
    out = subprocess.run(["bash", os.path.join(ROOT, "oracle", "build_ref.sh")], capture_output=True, text=True,
                         timeout=900, cwd=ROOT)
    if "no reference tree" in out.stdout:
        pytest.skip("the reference tree is not on this machine")
    assert out.returncode == 0, out.stdout[-2000:] + out.stderr[-2000:]
    assert os.path.exists(os.path.join(ROOT, "oracle", "_ref", "obj", "GpuLinearAlgebra.o"))
    exe = os.path.join(ROOT, "oracle", "_ref", "gpu_backend_check")
    if not os.path.exists(os.path.join(ROOT, "svfsiplus_gb300", "_build", "libsvgpu.so")):
        pytest.skip("libsvgpu.so not built: the link step needs it")
    run = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert run.returncode == 0 and "GpuLinearAlgebra linked" in run.stdout
