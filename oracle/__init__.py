"""CPU oracle (test infrastructure): float64 restatement of the reference path.

Only tests, the smoke check and the benchmark's CPU-baseline leg import this
package.  The ``oopao_gb300`` product never does.
"""
