"""CPU oracle for the TauFactor steady-state diffusion solve.

TEST INFRASTRUCTURE ONLY. Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline
leg of ``bench.py`` import this package, and only as the checker. The product package
``taufactor_gb300`` never imports, links or executes anything under ``oracle/``.

Modules
-------
``sor``         float32 restatement of the reference red-black SOR solve (taufactor/taufactor.py).
                Reproduces the reference's per-element arithmetic order, so a half-sweep is
                bitwise identical to the reference's on the same input.
``percolation`` restatement of the reference's spanning-cluster test
                (taufactor/metrics/connectivity.py:138-213) on scipy.ndimage.label.
``fp64``        FP64 "truth": the same discrete operator assembled in scipy.sparse and solved
                with preconditioned CG to a 1e-10 relative residual.
``ref_shim``    imports the reference package itself (only where its source tree exists) to
                pin the restatement; never used on the GPU machine.

Parity pins: ``tests/golden/*.npz`` hold outputs of the reference itself, produced by
``tests/golden/make_golden.py``; ``tests/test_oracle.py`` checks the restatement against them.
"""
