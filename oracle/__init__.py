"""CPU oracle for the tensor-train ALS hot path.

TEST INFRASTRUCTURE ONLY.  Nothing in the product package imports this
directory: only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py`` (its
``cpu_baseline`` leg and ``--impl reference`` arm) may use it, and only as the
checker or as the timed CPU baseline.

``oracle.tt_oracle`` restates, in plain NumPy/SciPy, the algorithm of
scikit_tt's ``solvers/sle.py`` (``als``), ``solvers/evp.py`` (``als``) and the
``TT`` operations they rely on (``tensor_train.py``).  Every function cites the
reference lines it follows.  The restatement is pinned against outputs of the
reference itself (``tests/golden/*.npz``, produced by
``tests/golden/make_golden.py`` from an import of the reference).
"""
