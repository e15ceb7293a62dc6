"""Run configuration: the parameter surface of the time step.

Field names, meanings and defaults follow ``NHQGConfig`` of the reference
(nhqg/config.py:9-108) so that a reference configuration constructs
unchanged.  The GPU engine covers ``float_dtype='float64'``,
``horizontal_dealiasing='23_rule'``, ``q_boundary='none'``,
``imex_scheme='ars222'`` and ``vertical_dealiasing='none'``; ``make_grid``
raises ``ValueError`` for other values, like the reference does for unknown
enums.
"""

from __future__ import annotations

import dataclasses


@dataclasses.dataclass(frozen=True)
class NHQGConfig:
    # resolution
    Nx: int = 256
    Nz: int = 32
    # physics
    Ra_tilde: float = 100.0
    sigma: float = 1.0
    beta: float = 0.0
    gamma: float = 0.0
    trap_r_star: float | None = None
    trap_sharpness: float = 20.0
    sponge_rate: float = 0.0
    sponge_r_start: float | None = None
    sponge_sharpness: float = 20.0
    Ld: float = float("inf")
    L: float = 20.0
    thermal_closure: str = "fixed_conduction"
    mean_temp_eps_sq: float = 1.0
    q_boundary: str = "none"
    w_bc_top: str = "dirichlet"
    nonlinear_advection: str = "jacobian"
    # time stepping
    dt: float = 1e-3
    t_final: float = 100.0
    imex_scheme: str = "ars222"
    # dissipation
    nu_q: float = 0.0
    hyper_order: int = 4
    nu_w: float = 0.0
    nu_theta: float = 0.0
    drag: float = 0.0
    # output
    save_interval: int = 100
    output_dir: str = "output"
    # numerics
    float_dtype: str = "float32"
    vertical_cutoff_n: int | None = None
    vertical_dealiasing: str = "none"
    horizontal_dealiasing: str = "32_rule"
    mean_exchange_discretization: str = "legacy"
    sbp_transfer_mode: str = "interp"
    sbp_corrector_substeps: int = 1
    imex_matmul_chunk: int = 0

    @property
    def Nk(self) -> int:
        return self.Nx // 2 + 1

    @property
    def Npad(self) -> int:
        return 3 * self.Nx // 2

    @property
    def dx(self) -> float:
        return self.L / self.Nx

    @property
    def Ld_inv_sq(self) -> float:
        return 0.0 if self.Ld == float("inf") else 1.0 / (self.Ld ** 2)

    @property
    def n_outputs(self) -> int:
        return int(self.t_final / self.dt) // self.save_interval

    def with_updates(self, **kwargs) -> "NHQGConfig":
        return dataclasses.replace(self, **kwargs)
