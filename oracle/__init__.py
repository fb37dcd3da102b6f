"""CPU oracle for the GraAda3D hot path -- TEST INFRASTRUCTURE ONLY.

``prism`` binds the C restatement of the reference's prism kernels
(``prism_oracle.c``); ``inversion`` restates the reference CGLS / Gauss-Newton
loop in NumPy; ``refbin`` runs the reference itself compiled into ``_ref/``
(available only where the reference sources are).  Only tests, the smoke
check and the benchmark's CPU-baseline leg use this package; the product path
in ``graada3d_gb300`` never imports it.
"""

import os as _os
import subprocess as _subprocess
from pathlib import Path as _Path


def reference_dir() -> _Path | None:
    """The reference tree the oracle recipe (``oracle/Makefile``) reads, or None
    where it is absent.  ``GRADA_REFERENCE`` overrides the recipe's default."""
    env = _os.environ.get("GRADA_REFERENCE")
    if env:
        ref = _Path(env)
    else:
        try:
            out = _subprocess.run(["make", "-s", "-C", str(_Path(__file__).resolve().parent), "refdir"],
                                  capture_output=True, text=True, check=True).stdout.strip()
        except (OSError, _subprocess.CalledProcessError):
            return None
        ref = _Path(out)
    return ref if (ref / "src" / "Forward_modelling" / "Fwd.h").exists() else None
