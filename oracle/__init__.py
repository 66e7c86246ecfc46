"""Oracle: a CPU restatement of the reference correlator.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` may import anything under ``oracle/``, and
only as the checker or the timed CPU baseline.  The product package
``powerfit_gb300`` never imports it and has no CPU fallback.

Contents
--------
``rotate_grid3d.c``   C restatement of ``_extensions.c:7-196`` (grid rotation).
``oracle.py``         numpy FP64 restatement of ``BaseCorrelator`` /
                      ``CPUCorrelator`` (``powerfitter.py:166-393``), the
                      ``_powerfit.pyx`` helpers and ``PowerFitter._combine``.
``build.py``          builds the C restatement, and (where the reference
                      sources are present) ``oracle/_ref`` from the reference's
                      own ``_extensions.c`` and ``_powerfit.pyx``.
``refimport.py``      imports the real reference correlator on top of
                      ``oracle/_ref`` to pin this restatement.

Parity pinning: ``tests/golden/make_golden.py`` runs the real reference and
commits its outputs as fixtures; ``tests/test_oracle_golden.py`` checks this
restatement against them.
"""
