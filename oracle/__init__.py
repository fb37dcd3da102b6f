"""CPU oracle for the GraAda3D hot path -- TEST INFRASTRUCTURE ONLY.

``prism`` binds the C restatement of the reference's prism kernels
(``prism_oracle.c``); ``inversion`` restates the reference CGLS / Gauss-Newton
loop in NumPy; ``refbin`` runs the reference itself compiled into ``_ref/``
(available only where the reference sources are).  Only tests, the smoke
check and the benchmark's CPU-baseline leg use this package; the product path
in ``graada3d_gb300`` never imports it.
"""
