"""fg_run_to_host: the TimeDisc loop with the state copied to the host during the last stage (the volume kernel of the
last stage over element chunks, each copied while the later ones compute) gives bitwise the state and times of fg_run
followed by fg_get_state. Cases cover every volume-kernel family and chunk shape: the shuffle-pair split kernel
(lines of 2 and 8 nodes: 16 and 1 elements per CTA, element counts that leave a partial last CTA), the per-node split
kernel on Gauss nodes, the weak-form kernel with 5 elements per CTA and the autotuner's 2-element variant, mortar
meshes, wall boundaries with the channel body force, an ensemble of two instances, and overintegration (each chunk
followed by its elements' filter kernel); calls of 1 and 3 steps, a call that continues the loop, and pinned host
memory."""
import numpy as np
import pytest

from _cases import perturb_state
from flexi_gb300 import mesh as fmesh, testcases
from flexi_gb300.solver import Flexi, make_config

pytestmark = pytest.mark.gpu

GAS = dict(kappa=1.4, R=71.42857, Pr=0.72, mu0=2e-3, CFLScale=0.9, DFLScale=0.9)
CASES = {
    "gl7_split_pi_hllc_br2": (dict(N=7, NodeType="gauss-lobatto", SplitDG="pi", Riemann="hllc", Lifting="br2"), "tgv4", None),
    "gl1_split_pi_roe_br1": (dict(N=1, NodeType="gauss-lobatto", SplitDG="pi", Riemann="roe", Lifting="br1"), "tgv5", None),
    "gauss5_split_pi_roeef_br1": (dict(N=5, NodeType="gauss", SplitDG="pi", Riemann="roeentropyfix", Lifting="br1"), "tgv3", None),
    "gauss2_weak_lf_br2": (dict(N=2, NodeType="gauss", SplitDG="weak", Riemann="lf", Lifting="br2"), "tgv5", None),
    "gauss5_weak_alt_shape": (dict(N=5, NodeType="gauss", SplitDG="weak", Riemann="roeentropyfix", Lifting="br1"), "tgv5", (1, 1, 2, 128)),
    "gl3_split_pi_mortar": (dict(N=3, NodeType="gauss-lobatto", SplitDG="pi", Riemann="roe", Lifting="br1"), "mortar", None),
    "gauss4_weak_channel": (dict(N=4, NodeType="gauss", SplitDG="weak", Riemann="roe", Lifting="br2", doTCSource=1, dpdx=-1.0), "channel",
                            None),
    "gauss3_weak_ensemble": (dict(N=3, NodeType="gauss", SplitDG="weak", Riemann="roe", Lifting="br1"), "ensemble", None),
    "gauss5_overint_cutoff": (dict(N=5, NodeType="gauss", SplitDG="weak", Riemann="roe", Lifting="br1", OverintegrationType=1, NUnder=3),
                              "tgv3", None),
    "gauss4_overint_conservative": (dict(N=4, NodeType="gauss", SplitDG="weak", Riemann="roeentropyfix", Lifting="br1",
                                         OverintegrationType=2, NUnder=2), "tgv4", None),
    "gauss11_overint_cutoff": (dict(N=11, NodeType="gauss", SplitDG="weak", Riemann="roeentropyfix", Lifting="br1", OverintegrationType=1,
                                    NUnder=7), "tgv2", None),
}


def _setup(name):
    kw, mesh, shapes = CASES[name]
    c = make_config(**dict(GAS, **kw))
    if mesh == "channel":
        m = fmesh.channel_box((3, 4, 2), beta=1.5, ngeo=2, t_wall=1.0, rho_wall=1.0, p_wall=1.0)
    elif mesh == "mortar":
        m = fmesh.mortar_box(4, perturb=0.05, seed=1)
    elif mesh == "ensemble":
        m = fmesh.concatenate([fmesh.tgv_box(2), fmesh.tgv_box(3, perturb=0.05, seed=3)])
    else:
        m = fmesh.tgv_box(int(mesh[3:]), ngeo=2, perturb=0.05, seed=1)
    pair = [Flexi(c, m), Flexi(c, m)]
    x = pair[0].elem_xgp()
    if mesh == "channel":
        U0 = testcases.channel_state(x, mach=0.1, kappa=c.kappa, R=c.R, t_wall=1.0, noise=0.05, seed=2)
    else:
        U0 = perturb_state(testcases.tgv_state(x, mach=0.2, kappa=c.kappa, R=c.R), seed=2)
    for f in pair:
        if shapes:
            f.set_launch_shapes(*shapes)
        f.U = U0
    return pair


@pytest.mark.parametrize("name", list(CASES))
def test_run_to_host_equals_run_then_get_state(name):
    f, g = _setup(name)
    for steps in (1, 3):
        t_f = f.TimeDisc(steps)
        U_f = f.U
        out = np.full(f.ushape, np.nan)
        t_g = g.TimeDisc_to_host_ptr(steps, out.ctypes.data)
        assert np.array_equal(t_f, t_g), (steps, t_f, t_g)
        assert np.array_equal(out, U_f), (steps, float(np.nanmax(np.abs(out - U_f))))
        # the device state is the step's state too
        assert np.array_equal(g.U, U_f)
    f.close()
    g.close()


def test_run_to_host_pinned_memory():
    torch = pytest.importorskip("torch")
    f, g = _setup("gl7_split_pi_hllc_br2")
    f.TimeDisc(2)
    U_f = f.U
    buf = torch.full((int(np.prod(f.ushape)),), float("nan"), dtype=torch.float64).pin_memory()
    g.TimeDisc_to_host_ptr(2, buf.data_ptr())
    assert np.array_equal(buf.numpy().reshape(f.ushape), U_f)
    # zero steps: the state as it is
    buf.fill_(float("nan"))
    g.TimeDisc_to_host_ptr(0, buf.data_ptr())
    assert np.array_equal(buf.numpy().reshape(f.ushape), U_f)
    f.close()
    g.close()
