"""The unmodified reference host (all of its sources except fft.c, matvec.c, iterative.c) links against the drop-in
layer + libadda_gb300 and runs up to the GPU: without a GPU it stops cleanly through the reference's own LogError.
Needs the reference sources (skipped elsewhere)."""
import os
import subprocess

import pytest

from conftest import ROOT, have_gpu
from oracle.oracle import ref_src_dir

REF_SRC = ref_src_dir()


@pytest.mark.skipif(not os.path.isdir(REF_SRC), reason="reference sources not present")
def test_reference_host_links_with_dropin(tmp_path, adda):
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "a-dda_gb300", "csrc", "dropin"), "REF_SRC=" + REF_SRC,
                    "-j8"], check=True)
    exe = os.path.join(ROOT, "a-dda_gb300", "_build", "adda_gb300")
    assert os.path.exists(exe)
    # prognosis: the reference host runs through InitDmatrix's accounting without touching the GPU
    p = subprocess.run([exe, "-grid", "16", "-prognosis", "-dir", str(tmp_path / "prog")], capture_output=True,
                       text=True, cwd=tmp_path)
    assert p.returncode == 0, p.stdout + p.stderr
    log = open(tmp_path / "prog" / "log").read()
    assert "The FFT grid is: 32x32x32" in log and "Total number of occupied dipoles: 2176" in log
    if not have_gpu():
        p = subprocess.run([exe, "-grid", "8", "-dir", str(tmp_path / "run")], capture_output=True, text=True,
                           cwd=tmp_path)
        assert p.returncode != 0
        assert "GPU initialisation failed" in p.stdout + p.stderr
        # surface mode: the drop-in evaluates the reflected tensor with the reference's ReflTerm_int (Sommerfeld
        # integrals of the reference's somnec) on the host before it reaches the GPU
        p = subprocess.run([exe, "-grid", "8", "-surf", "2", "2", "0.5", "-dir", str(tmp_path / "surf")],
                           capture_output=True, text=True, cwd=tmp_path)
        assert p.returncode != 0
        assert "GPU initialisation failed" in p.stdout + p.stderr
        assert "Reflected Green's tensor formulae: 'Sommerfeld integrals'" in open(tmp_path / "surf" / "log").read()
    # unsupported options stop with the reference's error path
    p = subprocess.run([exe, "-grid", "8", "-iter", "cgnr", "-prognosis", "-dir", str(tmp_path / "c")],
                       capture_output=True, text=True, cwd=tmp_path)
    assert p.returncode == 0  # prognosis stops before the solver
