"""CPU FP64 oracle for the voltax Newton inner loop -- TEST INFRASTRUCTURE ONLY.

This package restates, on the CPU in float64, what voltax computes on the
hot path, so the CUDA path can be checked against it:

* `devices`  -- device physics and local Jacobian blocks by forward-mode AD
  (voltax/elements/*.py, voltax/sparse.py:200-249)
* `stamp`    -- residual / Jacobian assembly in a fixed canonical order
  (voltax/circuit.py:209-226, voltax/sparse.py:220-249)
* `lu`       -- the padded per-bucket block-LDU factorization and solves
  (voltax/sparse.py:474-621)
* `analysis` -- damped Newton, gmin stepping, DC, BE/trapezoidal transient
  and the implicit-function adjoint (voltax/analysis.py:208-480)
* `plan`     -- numpy restatement of the symbolic planner (pivot groups,
  nested dissection, levels, buckets; voltax/sparse.py:257-535), the
  checker of the product's C++ planner; it builds the product's `Plan`
  container and reuses its `union_pairs` (the scipy matching that feeds
  both planners)
* `cvx.c` / `cbase` -- the compiled C restatement of the whole Newton loop
  (the timed CPU baseline) and its acceptance check of a given solution

It reads circuits by the reference's attribute names (``layout.groups``,
``elements[name].log_r``, ``.value``, ``.log_w``, ``.process.log_kp``, ...),
so apart from `plan` it does not import the product package. Only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may use
it; the product path never does.

Parity pins: the symbolic analysis the oracle factors with is pinned to the
reference's own output (tests/golden/symbolic.json, generated by running the
reference's voltax/sparse.py); the numeric restatement is pinned to the
reference's recorded RC-ladder values (voltax tests/test_analysis.py:33-49),
its EKV known answers (voltax tests/test_elements.py:188-220) and to dense
LAPACK / SuperLU solves. The reference's jax path itself cannot run here (no
jax), so summation order inside XLA's scatter-add is not pinned; the oracle
defines the canonical order (group, device, local row, local column).
"""
