"""The GANDALF-side drop-in subclass compiles against the reference's own headers.

include/gpu_gradh_sph_tree.hpp derives from the reference's GradhSphTree and overrides the
neighbour-search methods a Simulation calls; oracle/Makefile.ref's integration-check target
instantiates it for 3-D GradhSphParticle with -fsyntax-only.  Needs the reference sources
(GANDALF_SRC, or the upstream checkout of this container); skipped where they are absent.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("GANDALF_SRC", "/root/reference")


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "src", "Headers")), reason="reference sources absent")
@pytest.mark.skipif(shutil.which("g++") is None, reason="no g++")
def test_drop_in_subclass_compiles_against_reference_headers():
    res = subprocess.run(["make", "-s", "-f", os.path.join(ROOT, "oracle", "Makefile.ref"), f"REF={REF}",
                          "integration-check"], capture_output=True, text=True)
    assert res.returncode == 0, res.stdout + res.stderr
