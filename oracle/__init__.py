"""FP64 NumPy oracle for the PEPS evaluation path -- TEST INFRASTRUCTURE ONLY.

This package restates, in plain float64/complex128 NumPy + SciPy, the
algorithm of the reference package (fliingelephant/VMC, pure Python on JAX)
for the per-sample PEPS evaluation path: boundary-MPS strategies, the
sequential Metropolis transition, the estimate pass (O_k and E_loc), the
sliced QGT / SR solve and the time integrators.  Every function cites the
reference file:line it follows.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU baseline /
reference arm may import this package, and only as the checker or as the
timed CPU stand-in for the reference's JAX CPU path.  The GPU engine in
``vmc_gb300`` never imports it.

Pinning.  The reference cannot be executed here (jax, jaxlib, flax, netket and
plum are not installed and there is no network), and it ships no golden
vectors: all of its tests regenerate inputs from JAX seeds and check
properties.  The oracle is pinned by restating those property tests as
known-answer tests that do not depend on the reference's code:

* amplitudes and sliced gradients over all 2^9 configurations of a 3x3,
  D=4 PEPS against an independent brute-force contraction and exact
  multilinear derivatives (tests/test_peps_eval.py:18-77);
* central finite differences of the full gradient (tests/test_gradients_finite_diff.py:35-78);
* ZipUp / DensityMatrix / Variational == NoTruncation in the exact regime
  (tests/test_peps_strategy_equivalence.py:16-41);
* E_loc == (H psi)/psi with a dense H built independently with Kronecker
  products (tests/test_local_estimate_exact.py:24-79);
* sampled histograms against exact |psi|^2 (tests/test_sequential_sampling.py:126-208);
* MC energy / gradient against the exact full sum (tests/test_mc_energy_grad_evaluator.py:58-189);
* slice-ordering reorder and slice-vs-site SR solve (tests/test_qgt.py:84-160);
* solvers against dense solves (tests/test_qgt_solvers.py:15-46);
* RK4 / Euler against expm (tests/test_integrators.py:25-69);
* the first four again on random lattices, bond and physical dimensions (d = 2, 3), real and complex
  tensors and random Hermitian operators.

Truncated zip-up / variational amplitudes with ACTIVE truncation are pinned by
no reference test (the reference only checks the exact regime); for those the
oracle defines the answer with LAPACK ``gesdd`` / ``geqrf`` as the reference's
jaxlib 0.6.2 would, and comparisons flag samples whose singular-value gap at a
cut is too small for the kept subspace to be well defined.
"""
