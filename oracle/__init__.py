"""CPU oracle for the NHQG time-step hot path -- TEST INFRASTRUCTURE ONLY.

This package restates, in NumPy/SciPy, the reference algorithm of one NHQG
ARS(2,2,2) IMEX step (ksr-ocean/NHQG ``nhqg/grid.py``, ``nhqg/spectral.py``,
``nhqg/solver.py``); each function cites the reference ``file:line`` it
follows.  It is the checker: only ``tests/``, ``__graft_entry__.smoke()`` and
``bench.py``'s CPU-baseline / ``--impl reference`` legs may import it.  The
product package ``nhqg_gb300`` never imports it and has no CPU fallback.

Parity pin: the oracle is checked against golden vectors that the unmodified
reference source produced (``tests/golden/*.npz``, generator
``tests/golden/make_golden.py``) and against the reference's analytic
known-answer tests restated in ``tests/test_oracle_*.py``.
"""

from .nhqg_oracle import (  # noqa: F401
    OracleConfig,
    OracleGrid,
    OracleState,
    make_grid,
    explicit_rhs,
    explicit_rhs_dispatch,
    implicit_tendency,
    imex_implicit_solve,
    imex_mean_temp_solve,
    apply_balanced_sbp2_corrector,
    imex_step,
    sanitize_state,
    theta_perturbation_state,
    triple_conservative_flux_divergence_23,
    triple_jacobian_23,
    sponge_product_23,
    triple_conservative_flux_divergence_32,
    triple_jacobian_32,
    sponge_product_32,
    compute_diagnostics,
    DIAG_KEYS,
    DIAG_EXTRA_KEYS,
    energy_spectrum,
    vertical_mode_energy,
    high_mode_fraction,
    psi_ke_vertical_spectrum,
    shell_bin_index,
    spectra,
    shell_spectrum,
    field_shell_spectra,
)
