"""The drop-in translation units (graada3d_gb300/dropin/) compile against the
reference's unchanged class headers.  Needs the reference tree; skipped
elsewhere.  No GPU."""
import shutil
import subprocess
from pathlib import Path

import pytest

from conftest import REPO

from oracle import reference_dir

REF = reference_dir() or Path("missing-reference-tree")


@pytest.mark.skipif(not (REF / "src" / "Forward_modelling" / "Fwd.h").exists(),
                    reason="reference headers not available")
@pytest.mark.skipif(shutil.which("g++") is None, reason="no C++ compiler")
@pytest.mark.parametrize("unit", ["gb300_bridge", "Fwd_gb300", "GaussNewtonInversion_gb300",
                                  "InversionBase_gb300", "AdaptiveInversion_gb300",
                                  "FaceTable_gb300"])
def test_dropin_compiles_against_reference_headers(unit):
    lib = REF / "3rd_party_lib"
    cmd = ["g++", "-std=c++14", "-w", "-fsyntax-only",
           f"-I{lib / 'eigen'}", f"-I{lib / 'boost_1_72_0'}", f"-I{lib / 'Linterp'}",
           f"-I{lib / 'Timer'}", f"-I{REF / 'src' / 'Forward_modelling'}",
           f"-I{REF / 'src' / 'Inversion'}", f"-I{REPO / 'oracle' / 'gsl_stub'}",
           str(REPO / "graada3d_gb300" / "dropin" / f"{unit}.cpp")]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
