"""CPU oracle for the WesterveltEDG.jl right-hand side and RK4 hot path.

TEST INFRASTRUCTURE ONLY. Nothing in the product package may import, call,
link or execute anything in this directory; only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline legs of ``bench.py`` use it,
and only as the checker (or as the timed CPU port of the reference).

Contents, each a restatement of the reference's algorithm (WesterveltEDG.jl
v0.3.0, Julia; the reference cannot be run here because no Julia toolchain is
available):

* ``quadrature.py``    -- ``src/quadrature.jl`` (Jacobi polynomials, Golub-Welsch)
* ``coefficients.py``  -- ``src/coefficients.jl``
* ``precompute.py``    -- ``src/solver.jl:16-68, 341-770`` (``precompute``,
                          ``_side_values!``, ``_rhs_data``)
* ``rhs_oracle.c``     -- ``src/rhs.jl:65-951`` (batched RHS, Chebyshev and CG
                          mass solves) and ``src/solver.jl:278-321, 864-888``
                          (RK4, energy diagnostics), plain C + OpenMP
* ``rhs.py``           -- ctypes binding of ``rhs_oracle.c``
* ``solver.py``        -- ``src/solver.jl:167-228, 772-836, 892-958`` (``solve``,
                          error norms, ``difference_norms``, source-mode run)
* ``reference_rhs.py`` -- ``test/reference_rhs.jl`` (the dense element-by-element
                          RHS of v0.1.0) with the ``dense_volume`` /
                          ``reference_pre`` adaptors of ``test/runtests.jl:11-20,
                          233-239``: the independent second implementation

Parity pins: the oracle is checked against the reference's stored results
(``test/runtests.jl:207-217``, ``data/convergence/results.csv``,
``data/alpha_limit/order.csv``, ``data/steepening/*``; fixtures in
``tests/golden/``) and against its own dense second implementation on the
reference's differential test grid (``test/runtests.jl:189-293``).
"""
