"""CPU oracle for the restarted-PDHG LP path — TEST INFRASTRUCTURE ONLY.

Nothing in the product imports this package.  Only ``tests/``,
``__graft_entry__.smoke()`` (as the checker) and the CPU-baseline legs of
``bench.py`` use it.

Contents
--------
``pdhg_ref``   FP64 NumPy/SciPy restatement of the reference's restarted PDHG
               (``solver/lp/pdhg.py:62-259``): standard-form conversion, fixed
               diagonal step sizes, θ = 1 extrapolation, ergodic averaging,
               KKT check every 50 iterations, restart-to-average on halving.
               Pinned against golden vectors produced by the reference itself
               (``tests/golden/``), including the reference's published Netlib
               rows (``benchmarks/results/benchmark_comparison.csv:5,9,13,17``).
``kkt``        FP64 KKT evaluators: the reference's standard-form error
               (``pdhg.py:184-196``) for any box-form primal/dual pair, and the
               box-form relative KKT the GPU engine reports.
``pdlp_ref``   FP64 restatement of the GPU engine's adaptive ("PDLP") mode, for
               step-by-step comparison on small problems.
``simplex``    FP64 bounded revised simplex (two phases, dense LU), the objective
               oracle; matches the reference simplex on every golden problem.
``gnn_ref``    FP64 restatement of the warm-start network (forward, backward).
``pdhg_ref.c`` C + OpenMP restatement of ``pdhg_ref`` used as the timed CPU
               baseline (all host threads).
"""
