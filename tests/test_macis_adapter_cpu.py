"""The C++ adapter of MACIS's interfaces (include/qdkgb_macis_generator.hpp)
compiles against the reference's own headers and links against libqdkgb.so:
GpuHamiltonianGenerator<wfn_t<64>> and <wfn_t<128>> implement every pure
virtual of macis::HamiltonianGenerator, and GpuSparseOperator fits
macis::davidson.  The reference's headers need the project's API shims
(oracle/ref_shims) and its base.cxx; the test is skipped where the reference
checkout is absent (QDK_REFERENCE names it; else a checkout named
"reference" beside the repository is used)."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

REFERENCE = os.environ.get("QDK_REFERENCE") or os.path.join(os.path.dirname(os.path.abspath(ROOT)), "reference")
MACIS = os.path.join(REFERENCE, "external", "macis")


@pytest.mark.skipif(not os.path.isdir(os.path.join(MACIS, "include", "macis")), reason="reference checkout absent")
def test_adapter_compiles_links_and_runs(pkg, tmp_path):
    lib = pkg.build.build()
    gxx = shutil.which("g++")
    assert gxx
    inc = ["-I" + os.path.join(ROOT, "oracle", "ref_shims"), "-I" + os.path.join(MACIS, "include"),
           "-I" + os.path.join(MACIS, "src", "sparsexx", "include"),
           "-I" + os.path.join(MACIS, "src", "lobpcgxx", "include"), "-I" + os.path.join(ROOT, "include")]
    flags = ["-std=c++20", "-O1", "-fopenmp", "-w"]
    base = str(tmp_path / "base.o")
    subprocess.run([gxx, *flags, *inc, "-c", os.path.join(MACIS, "src", "macis", "hamiltonian_generator", "base.cxx"),
                    "-o", base], check=True, capture_output=True, text=True)
    exe = str(tmp_path / "adapter_check")
    r = subprocess.run([gxx, *flags, *inc, os.path.join(ROOT, "tests", "cpp", "macis_adapter_check.cpp"), base,
                        lib, "-Wl,-rpath," + os.path.dirname(lib), "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr[-2000:]
    assert out.stdout.startswith("no device: qdkgb:") or out.stdout.startswith("device: nnz"), out.stdout
