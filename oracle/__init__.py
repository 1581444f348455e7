"""CPU oracle for the effective-Hamiltonian hot path of MPSKit.jl (v0.13.13).

TEST INFRASTRUCTURE ONLY.  Nothing in the product (the `mpsgb` package, its C-ABI
library or its kernels) may import, call or link this package.  It is imported by
`tests/`, by `__graft_entry__.smoke()` (as the checker) and by the `cpu_baseline`
leg and `--impl reference` arm of `bench.py`.

The oracle is a plain numpy FP64 restatement of the reference algorithm.  Each
function cites the reference file:line it follows (paths relative to the MPSKit.jl
project root).  The reference itself is Julia and cannot run in this environment
(no Julia toolchain), and the arithmetic of the reference lives in non-vendored
Julia packages (TensorKit 0.17.1, TensorOperations 5.6.2, BlockTensorKit 0.3.15,
KrylovKit 0.8-0.10, MatrixAlgebraKit 0.6.5).  The oracle restates their published
algorithms (tensor contraction by index string; Lanczos / Krylov-Schur eigsolve;
truncated SVD) and is pinned by:

  * the reference's own known-answer tests (TFIM L=4 doctest energy -4.7588,
    `src/algorithms/groundstate/find_groundstate.jl:49-64`; spin-1/2 Heisenberg
    L=20 energy -8.6824724, `test/algorithms/groundstate.jl:151-175`),
  * exact diagonalisation built directly from the lattice terms (independent of
    the MPO builder), and
  * closed forms (free-fermion TFIM, Bethe-ansatz Heisenberg energy density).

Tensors are numpy arrays whose axes follow TensorKit's leg order
(codomain legs, then domain legs): MPS tensor A[l, s, r], MPO tensor W[wl, s, s', wr]
(dense over the MPO channel sum space, channel 0 = "not started", last = "finished"),
left environment GL[a, w, a'], right environment GR[b', w, b], two-site tensor
x[l, s1, r, s2].
"""
