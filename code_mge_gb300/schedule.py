"""Work accounting of one multigrid cycle (solver.f90:127-234).

Mirrors the cycle scheduler to count, per level, the euler update calls
(the unit of the benchmark metric: one physical cell advanced by one full
RK update is one cell-update) and the residual-only calls.
"""


def cycle_visits(nlevel, mgtype, mlvl=None):
    """(updates[level], residuals[level]) of one cycle at FMG level mlvl, 1-based levels."""
    mlvl = nlevel if mlvl is None else mlvl
    upd = [0] * (nlevel + 2)
    res = [0] * (nlevel + 2)
    icyc = [0] * (nlevel + 2)
    mgl = mlvl
    while True:  # lopmg
        while True:  # lopr
            icyc[mgl] += 1
            upd[mgl] += 1
            if mlvl == 1:
                return upd, res
            res[mgl] += 1
            mgl -= 1
            if mgl == 1:
                break
        while True:  # lopp
            upd[mgl] += 1
            mgl += 1
            if mgl == mlvl:
                return upd, res
            if icyc[mgl] != mgtype:
                break
            icyc[mgl] = 0


def cell_updates_per_cycle(case, mlvl=None):
    nlevel = case.prm.nlevel
    upd, _ = cycle_visits(nlevel, case.prm.mgtype, mlvl)
    cells = case.cells_per_level()
    return sum(cells[L - 1] * upd[L] for L in range(1, nlevel + 1))


def residual_cells_per_cycle(case, mlvl=None):
    nlevel = case.prm.nlevel
    _, res = cycle_visits(nlevel, case.prm.mgtype, mlvl)
    cells = case.cells_per_level()
    return sum(cells[L - 1] * res[L] for L in range(1, nlevel + 1))
