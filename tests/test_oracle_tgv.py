"""End-to-end pin of the CPU oracle: FLEXI's Taylor-Green regression references
regressioncheck/checks/tgv/split (GL N=7) and tgv/splitGauss (Gauss N=5: split form with
entropy-variable prolongation and the split-Gauss surface integral), both split PI, RoeEntropyFix, BR1,
8^3 periodic, CFL=DFL=0.8, and tgv/oInt (Gauss N=11, weak form, overintegration by the modal cut-off
filter to NUnder=7, 4^3, CFL=DFL=0.9), all at Re=1600, Ma=0.1, R=71.42857. Their TGVAnalysis CSV rows are written every 10
steps and compared by the reference at 1e-4 relative (analyze.ini). Checks the t=0 row and the first rows
after stepping with the reference's time-step control (UpdateTimeStep/CALCTIMESTEP), including the time
column."""
import numpy as np
import pytest

from flexi_gb300 import mesh as fmesh
from oracle import oracle as orc

TGV_CFG = dict(N=7, nodeType=orc.NT_GL, riemann=33, riemannBC=-1, lifting=1, weakLifting=0, consLifting=0, splitDG=4,
               etaBR2=2.0, etaBR2_wall=-1.0, kappa=1.4, R=71.42857, Pr=0.72, mu0=6.25e-4, CFLScale=0.8, DFLScale=0.8,
               doTCSource=0, dpdx=-1.0)
TGV_GAUSS_CFG = dict(TGV_CFG, N=5, nodeType=orc.NT_GAUSS)
REL = 1e-4
# tgv/oInt: N=11 Gauss, weak form, overintegration by the modal cut-off filter to NUnder=7, 4^3, CFL=DFL=0.9
TGV_OINT_CFG = dict(TGV_CFG, N=11, nodeType=orc.NT_GAUSS, splitDG=-1, CFLScale=0.9, DFLScale=0.9, overintType=1, NUnder=7)
CASES = {"split": ("tgv_reference", TGV_CFG, 8), "splitGauss": ("tgv_splitgauss_reference", TGV_GAUSS_CFG, 8),
         "oInt": ("tgv_oint_reference", TGV_OINT_CFG, 4)}


def tgv_oracle(n=8, cfg=TGV_CFG):
    m = fmesh.tgv_box(n, ngeo=1)
    o = orc.Oracle(cfg, m)
    x = o.mesh_array("Elem_xGP")
    o.set_state(orc.tgv_exact(x, mach=0.1, kappa=cfg["kappa"], R=cfg["R"]))
    o.overintegrate_state()  # timedisc.f90:115-123 (no-op without overintegration)
    return o


def analysis(o, cfg=TGV_CFG):
    return orc.tgv_analysis(cfg["N"], cfg["nodeType"], o.mesh_array("sJ"), o.get_state(), o.gradients(), 10, cfg["kappa"], cfg["R"],
                            cfg["mu0"])


def compare_row(row, ref, scale):
    # relative 1e-4 on every column; columns at round-off level (|ref| < 1e-12 of the column scale) in absolute terms
    for c in range(len(ref)):
        if abs(ref[c]) > 1e-12 * scale[c]:
            assert abs(row[c] - ref[c]) <= REL * abs(ref[c]), (c, row[c], ref[c])
        else:
            assert abs(row[c]) <= 1e-9 * scale[c], (c, row[c], ref[c])


@pytest.mark.parametrize("case", list(CASES))
def test_tgv_t0_row(case, request):
    fixture, cfg, ne = CASES[case]
    _, rows = request.getfixturevalue(fixture)
    o = tgv_oracle(ne, cfg=cfg)
    o.time_derivative(0.0)
    a = analysis(o, cfg)
    scale = np.abs(rows[:, 1:]).max(axis=0)
    compare_row(a, rows[0, 1:], scale)


@pytest.mark.timeout(900)
@pytest.mark.parametrize("case", list(CASES))
def test_tgv_first_rows(case, request):
    fixture, cfg, ne = CASES[case]
    _, rows = request.getfixturevalue(fixture)
    o = tgv_oracle(ne, cfg=cfg)
    scale = np.abs(rows[:, 1:]).max(axis=0)
    t = 0.0
    o.time_derivative(0.0)
    for r in (1, 2):
        for _ in range(10):
            dt, err = o.calc_timestep()
            assert err == 0
            t = o.timestep(t, dt)
        assert abs(t - rows[r, 0]) <= 1e-10 * rows[r, 0], (t, rows[r, 0])
        compare_row(analysis(o, cfg), rows[r, 1:], scale)
