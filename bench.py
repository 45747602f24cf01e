"""Benchmark: FP64 DOF*stage/s of FLEXI's DGSEM Navier-Stokes RHS + LSERK stepper on GB300.

Workload (default): Taylor-Green vortex on a curved periodic 32^3 hexahedral mesh, N=7 Gauss-Lobatto,
split form with the Pirozzoli flux, BR2 lifting, HLLC surface flux (--riemann roeentropyfix selects the
surface flux of the reference's own split-form TGV regression; the reference rejects HLLC with the split
form, the CPU restatement and these kernels do not), Re=1600, Ma=0.1, FP64, CarpenterRK4-5 with CFL/DFL
time step control at CFLScale=DFLScale=0.8 (the setting of the reference's split-form TGV regression;
0.9 is at the stability edge of this discretisation). 16.8 M DOF x 5 variables; the state alone (671 MB) exceeds L2 (129 MB), so no L2 flush is
needed between steps. Synthetic data: mesh and initial state are generated (no external dataset).

value  : DOF*stage/s on the device, inputs resident in HBM, K steps bracketed by CUDA events on the
         solver's stream (barrier + synchronize on both sides, max over ranks).
e2e    : the same metric through the public C ABI with the state in pinned host memory: each step
         uploads U (fg_set_state), advances one step (fg_run), downloads U (fg_get_state).
--workload tgv-splitgauss : the discretisation of the reference's tgv/splitGauss regression (N=5 Gauss, split
         PI with entropy-variable prolongation and the split-Gauss surface integral, BR1, RoeEntropyFix) on a
         curved 40^3 mesh (13.8 M DOF), same metric and timing.
--workload tgv-oint : the discretisation of the reference's tgv/oInt regression (N=11 Gauss, weak form,
         overintegration by the modal cut-off of J u_t to NUnder=7, BR1, RoeEntropyFix, CFL=DFL=0.9) on a
         curved 16^3 mesh (7.1 M DOF), same metric and timing.
--workload tgv-mortar : TGV on a periodic box with mortar interfaces (24^3 cells whose z-layers alternate
         between one element per cell and 2x2 elements, 34560 elements, 13824 mortars 1->4, perturbed,
         NGeo=1), N=7 Gauss-Lobatto, split PI, BR1 (the lifting the mortar path supports), RoeEntropyFix
         (17.7 M DOF), same metric and timing.
--impl reference : the CPU implementation of the path (the C++ restatement of FLEXI's Fortran solver,
         FLEXI itself cannot be built here: Fortran/MPI/HDF5) on all host threads, bounded sample per step.
Multi-GPU: the path does not shard on this setup (no halo exchange is built); N ranks run N replicas.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "FP64 DOF*stage/s (N=7 TGV)"
UNIT = "DOF*stage/s"
# algorithmic flops per DOF and RK stage of the reference algorithm (counted with the oracle's
# flop-counting scalar on this configuration; pinned by tests/test_bench_constants.py)
FLOPS_PER_DOF_STAGE = {"prep": 24.5, "lift": 322.5, "vol": 1408.9}
FLUX_FLOPS_PER_DOF_STAGE = {"hllc": 107.6, "roeentropyfix": 145.5}
RIEMANN_IDS = {"hllc": 2, "roeentropyfix": 33}
RIEMANN_NAMES = {"hllc": "HLLC", "roeentropyfix": "RoeEntropyFix"}


# the Gauss split form (N=5, split PI with entropy-variable prolongation and the split-Gauss surface
# integral, BR1, RoeEntropyFix: the discretisation of the reference's tgv/splitGauss regression)
SPLITGAUSS_METRIC = "FP64 DOF*stage/s (N=5 TGV, Gauss split form)"
SPLITGAUSS_FLOPS_PER_DOF_STAGE = {"prep": 128.0, "lift": 500.0, "flux": 194.0, "vol": 1750.5}
# overintegration (the discretisation of the reference's tgv/oInt regression: N=11 Gauss, weak form, BR1,
# RoeEntropyFix, modal cut-off filter of J u_t to NUnder=7); "vol" includes the filter
OINT_METRIC = "FP64 DOF*stage/s (N=11 TGV, overintegration cut-off to NUnder=7)"
OINT_FLOPS_PER_DOF_STAGE = {"prep": 78.5, "lift": 640.0, "flux": 94.75, "vol": 935.25}
# mortar interfaces (N=7 Gauss-Lobatto, split PI, BR1, RoeEntropyFix on the periodic mortar box); the
# oracle books U_Mortar in prep, the lifting projections in lift and the small-side fluxes with Flux_Mortar
# in flux, the GPU runs them in k_mortar_pre / k_mortar_face
MORTAR_METRIC = "FP64 DOF*stage/s (N=7 TGV, mortar box)"
MORTAR_FLOPS_PER_DOF_STAGE = {"prep": 49.8, "lift": 398.4, "flux": 198.2, "vol": 1409.25}


def flops_per_dof_stage(riemann, kind="tgv"):
    if kind == "tgv-splitgauss":
        return dict(SPLITGAUSS_FLOPS_PER_DOF_STAGE)
    if kind == "tgv-oint":
        return dict(OINT_FLOPS_PER_DOF_STAGE)
    if kind == "tgv-mortar":
        return dict(MORTAR_FLOPS_PER_DOF_STAGE)
    return dict(FLOPS_PER_DOF_STAGE, flux=FLUX_FLOPS_PER_DOF_STAGE[riemann])
# compulsory HBM traffic per DOF and stage: U read+write, Ut_tmp read+write, 9 metric terms + sJ
BYTES_ALG_PER_DOF_STAGE = 240.0
# HBM copy bandwidth of a GB300 when no measured figure is present on the box (one earlier measurement)
HBM_FALLBACK_GBS = 6800.0


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--elems", type=int, default=None, help="elements per direction (tgv: 32, tgv-splitgauss: 40, tgv-oint: 16)")
    p.add_argument("--riemann", default="hllc", choices=sorted(RIEMANN_IDS), help="surface Riemann solver")
    p.add_argument("--workload", default="tgv", choices=["tgv", "tgv-splitgauss", "tgv-oint", "tgv-mortar", "ensemble", "adjoint",
                                                        "adjoint-channel"],
                   help="tgv: the single-case N=7 TGV; tgv-splitgauss: the N=5 Gauss split form of the reference's tgv/splitGauss "
                        "regression on a curved 40^3 mesh; tgv-oint: the N=11 overintegration of tgv/oInt on a curved 16^3 mesh; "
                        "tgv-mortar: N=7 on a 24^3-cell box with 1->4 mortar interfaces; ensemble: 256 independent TGV/vortex instances at N=5 against a loop over "
                        "instances; adjoint: gradient of a kinetic-energy loss over a 200-step TGV solve (16^3, N=5)")
    p.add_argument("--ckpt", type=int, default=20, help="adjoint: checkpoint interval in steps")
    p.add_argument("--fd-dirs", type=int, default=20, help="adjoint: random directions of the finite-difference check")
    p.add_argument("--exact-dirs", type=int, default=3, help="adjoint: directions (the first of the FD check) whose exact tangent "
                                                              "the oracle also computes (dual numbers, host threads)")
    p.add_argument("--instances", type=int, default=256, help="ensemble size")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu-baseline", action="store_true", help="skip the CPU baseline leg (profiling runs)")
    a = p.parse_args()
    if a.elems is None:
        a.elems = {"tgv-splitgauss": 40, "tgv-oint": 16, "tgv-mortar": 24}.get(a.workload, 32)
    if a.workload in ("tgv-splitgauss", "tgv-oint", "tgv-mortar"):
        a.riemann = "roeentropyfix"
    return a


def workload_config(n, riemann, kind="tgv"):
    if kind == "tgv-mortar":
        ne = 5 * n ** 3 // 2
        dof = ne * 512
        return {"workload": f"TGV on the periodic mortar box of {n}^3 cells (z-layers alternating 1 and 2x2 elements per cell, "
                            f"{ne} elements, {n ** 3} mortars 1->4, perturbation 0.05, NGeo=1), N=7 Gauss-Lobatto, split PI, BR1, "
                            f"RoeEntropyFix, FP64",
                "n_elems": ne, "n_mortars": n ** 3, "N": 7, "dof": dof, "Re": 1600, "Ma": 0.1, "CFLScale": 0.8, "DFLScale": 0.8,
                "time_integration": "CarpenterRK4-5, 5 stages/step, CFL/DFL dt each step",
                "l2": f"inputs larger than L2 (state {dof * 40 / 1e6:.0f} MB)", "parallelism": "replicas"}
    if kind == "tgv-oint":
        dof = n ** 3 * 1728
        return {"workload": f"TGV {n}^3 curved (perturbation 0.05, NGeo=3), N=11 Gauss, weak form, overintegration by the modal "
                            f"cut-off filter of J u_t to NUnder=7, BR1, RoeEntropyFix, FP64",
                "n_elems": n ** 3, "N": 11, "dof": dof, "Re": 1600, "Ma": 0.1, "CFLScale": 0.9, "DFLScale": 0.9,
                "time_integration": "CarpenterRK4-5, 5 stages/step, CFL (on NUnder) / DFL dt each step",
                "l2": f"inputs larger than L2 (state {dof * 40 / 1e6:.0f} MB)", "parallelism": "replicas"}
    if kind == "tgv-splitgauss":
        dof = n ** 3 * 216
        return {"workload": f"TGV {n}^3 curved (perturbation 0.05, NGeo=3), N=5 Gauss, split PI with entropy-variable prolongation "
                            f"and the split-Gauss surface integral, BR1, RoeEntropyFix, FP64",
                "n_elems": n ** 3, "N": 5, "dof": dof, "Re": 1600, "Ma": 0.1, "CFLScale": 0.8, "DFLScale": 0.8,
                "time_integration": "CarpenterRK4-5, 5 stages/step, CFL/DFL dt each step",
                "l2": f"inputs larger than L2 (state {dof * 40 / 1e6:.0f} MB)", "parallelism": "replicas"}
    return {"workload": f"TGV {n}^3 curved (perturbation 0.05, NGeo=3), N=7 Gauss-Lobatto, split PI, BR2, {RIEMANN_NAMES[riemann]}, FP64",
            "n_elems": n ** 3, "N": 7, "dof": n ** 3 * 512, "Re": 1600, "Ma": 0.1, "CFLScale": 0.8, "DFLScale": 0.8,
            "time_integration": "CarpenterRK4-5, 5 stages/step, CFL/DFL dt each step",
            "l2": "inputs larger than L2 (state 671 MB at 32^3)", "parallelism": "replicas"}


def solver_config(riemann, kind="tgv"):
    from flexi_gb300.solver import make_config
    if kind == "tgv-mortar":
        return make_config(N=7, NodeType="gauss-lobatto", SplitDG="pi", Riemann="roeentropyfix", Lifting="br1", kappa=1.4, R=71.42857,
                           Pr=0.72, mu0=6.25e-4, CFLScale=0.8, DFLScale=0.8)
    if kind == "tgv-oint":
        return make_config(N=11, NodeType="gauss", SplitDG="weak", Riemann="roeentropyfix", Lifting="br1", kappa=1.4, R=71.42857,
                           Pr=0.72, mu0=6.25e-4, CFLScale=0.9, DFLScale=0.9, OverintegrationType=1, NUnder=7)
    if kind == "tgv-splitgauss":
        return make_config(N=5, NodeType="gauss", SplitDG="pi", Riemann="roeentropyfix", Lifting="br1", kappa=1.4, R=71.42857,
                           Pr=0.72, mu0=6.25e-4, CFLScale=0.8, DFLScale=0.8)
    return make_config(N=7, NodeType="gauss-lobatto", SplitDG="pi", Riemann=riemann, Lifting="br2", kappa=1.4, R=71.42857,
                       Pr=0.72, mu0=6.25e-4, CFLScale=0.8, DFLScale=0.8)


def oracle_config(riemann, kind="tgv"):
    """The same discretisation for the CPU restatement."""
    if kind == "tgv-mortar":
        return dict(N=7, nodeType=2, riemann=33, riemannBC=-1, lifting=1, weakLifting=0, consLifting=0, splitDG=4, etaBR2=2.0,
                    etaBR2_wall=-1.0, kappa=1.4, R=71.42857, Pr=0.72, mu0=6.25e-4, CFLScale=0.8, DFLScale=0.8, doTCSource=0, dpdx=-1.0)
    if kind == "tgv-oint":
        return dict(N=11, nodeType=1, riemann=33, riemannBC=-1, lifting=1, weakLifting=0, consLifting=0, splitDG=-1, etaBR2=2.0,
                    etaBR2_wall=-1.0, kappa=1.4, R=71.42857, Pr=0.72, mu0=6.25e-4, CFLScale=0.9, DFLScale=0.9, doTCSource=0, dpdx=-1.0,
                    overintType=1, NUnder=7)
    if kind == "tgv-splitgauss":
        return dict(N=5, nodeType=1, riemann=33, riemannBC=-1, lifting=1, weakLifting=0, consLifting=0, splitDG=4, etaBR2=2.0,
                    etaBR2_wall=-1.0, kappa=1.4, R=71.42857, Pr=0.72, mu0=6.25e-4, CFLScale=0.8, DFLScale=0.8, doTCSource=0, dpdx=-1.0)
    return dict(N=7, nodeType=2, riemann=RIEMANN_IDS[riemann], riemannBC=-1, lifting=2, weakLifting=0, consLifting=0, splitDG=4, etaBR2=2.0,
                etaBR2_wall=-1.0, kappa=1.4, R=71.42857, Pr=0.72, mu0=6.25e-4, CFLScale=0.8, DFLScale=0.8, doTCSource=0, dpdx=-1.0)


def metric_name(kind):
    return {"tgv-splitgauss": SPLITGAUSS_METRIC, "tgv-oint": OINT_METRIC, "tgv-mortar": MORTAR_METRIC}.get(kind, METRIC)


def workload_mesh(kind, n, seed=0):
    """The workload's mesh: the curved TGV box, or the periodic mortar box."""
    from flexi_gb300 import mesh as fmesh
    if kind == "tgv-mortar":
        return fmesh.mortar_box(n, perturb=0.05, seed=seed)
    return fmesh.tgv_box(n, ngeo=3, perturb=0.05, seed=seed)


def kernel_names(kind):
    if kind == "tgv-oint":
        return {"vol": "k_vol_weak<12,Gauss> + k_overint<12>", "lift": "k_lift<12,Gauss>", "flux": "k_flux<12>", "prep": "k_prep<12,Gauss>"}
    if kind == "tgv-splitgauss":
        return {"vol": "k_vol_split_gen<6,Gauss>", "lift": "k_lift<6,Gauss>", "flux": "k_flux<6>", "prep": "k_prep<6,Gauss>"}
    if kind == "tgv-mortar":
        return {"vol": "k_vol_split<8>", "lift": "k_lift<8,GL,MORTAR>", "flux": "k_flux<8>", "prep": "k_prep<8,GL>",
                "other": "k_mortar_pre<8> + k_mortar_face<8>"}
    return {"vol": "k_vol_split<8>", "lift": "k_lift<8,GL>", "flux": "k_flux<8>", "prep": "k_prep<8,GL>"}


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown," \
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                                          "-i", str(self.gpu)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"), f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


def ncu_traffic(kind="tgv"):
    """DRAM bytes per DOF of each kernel class from the committed ncu summary (key: workload)."""
    try:
        t = json.load(open(os.path.join(ROOT, "profiles", "traffic.json")))
    except Exception:
        return {}
    return t.get(kind, {}) if kind != "tgv" else {k: v for k, v in t.items() if not isinstance(v, dict)}


def fp64_instr(kind="tgv"):
    """Executed FP64 instructions per DOF of each kernel class (committed ncu counts, profiles/fp64_instr.json)."""
    try:
        return json.load(open(os.path.join(ROOT, "profiles", "fp64_instr.json"))).get(kind, {})
    except Exception:
        return {}


def fp64_roofline(instr, dof, launch_s, n_sm, sm_hz, probe):
    """Roofline of an FP64-issue-bound launch. The FP64 pipe's nominal rate (the 100 % of ncu's
    sm__pipe_fp64_cycles_active) is 2 thread-instructions per clock per SM; achieved = the launch's executed DADD/DMUL/DFMA
    flops (DFMA = 2; ncu counts per DOF x DOF) per CUDA-event launch time, peak = the nominal rate for the same instruction
    mix, frac = achieved / peak. The probe (fg_probe_fp64_pipe: independent chains of one operation on every SM) gives the
    rate an arithmetic FP64 stream attains, reported as a fraction of the nominal rate next to it."""
    n_instr = instr["dadd"] + instr["dfma"] + instr["dmul"]
    flops_per_instr = (instr["dadd"] + instr["dmul"] + 2.0 * instr["dfma"]) / n_instr
    nominal = 2.0 * n_sm * sm_hz  # thread-instructions per second
    instr_rate = n_instr * dof / launch_s
    attainable = max(probe.values()) * 1e12
    return {"achieved": instr_rate * flops_per_instr / 1e12, "peak": nominal * flops_per_instr / 1e12, "frac": instr_rate / nominal,
            "fp64_instr_per_s": instr_rate, "nominal_fp64_instr_per_s": nominal, "attainable_fp64_instr_per_s": attainable,
            "attainable_frac_of_nominal": attainable / nominal, "frac_of_attainable": instr_rate / attainable}


def cpu_baseline_sample(riemann, n_elems_dir=32, budget_s=12.0, kind="tgv"):
    """Oracle (C++ restatement of FLEXI's operator) on all host threads: the workload's own mesh and
    discretisation, timed RK steps until the budget is used (at least two). Returns (DOF*stage/s, threads, sample)."""
    import numpy as np
    from flexi_gb300 import mesh as fmesh, testcases
    from oracle import oracle as orc
    orc.set_threads(os.cpu_count() or 1)
    cfg = oracle_config(riemann, kind)
    m = workload_mesh(kind, n_elems_dir)
    o = orc.Oracle(cfg, m)
    o.set_state(testcases.tgv_state(o.mesh_array("Elem_xGP"), mach=0.1, kappa=1.4, R=71.42857))
    o.overintegrate_state()  # timedisc.f90:115-123 (no-op without overintegration)
    dof = m.n_elems * (cfg["N"] + 1) ** 3
    t = 0.0
    dt, _ = o.calc_timestep()
    t = o.timestep(t, dt)  # warm-up
    steps, t0 = 0, time.perf_counter()
    while True:
        dt, _ = o.calc_timestep()
        t = o.timestep(t, dt)
        steps += 1
        el = time.perf_counter() - t0
        if (el >= budget_s and steps >= 2) or steps >= 200:
            break
    rate = dof * 5 * steps / el
    return rate, orc.max_threads(), f"{m.description}, same discretisation ({dof} DOF), {steps} RK steps with dt control, {el:.1f} s"


def run_reference(args):
    ws, rank, _ = dist_info()
    if rank != 0:
        return
    import numpy as np
    from flexi_gb300 import mesh as fmesh, testcases
    from oracle import oracle as orc
    threads = os.cpu_count() or 1
    orc.set_threads(threads)
    cfg = oracle_config(args.riemann, args.workload)
    m = workload_mesh(args.workload, args.elems)  # the workload's own mesh; each step is one RK step of it
    o = orc.Oracle(cfg, m)
    o.set_state(testcases.tgv_state(o.mesh_array("Elem_xGP"), mach=0.1, kappa=1.4, R=71.42857))
    o.overintegrate_state()  # timedisc.f90:115-123 (no-op without overintegration)
    dof = m.n_elems * (cfg["N"] + 1) ** 3
    t = 0.0
    for _ in range(args.warmup):
        dt, _ = o.calc_timestep()
        t = o.timestep(t, dt)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        dt, _ = o.calc_timestep()
        t = o.timestep(t, dt)
    el = time.perf_counter() - t0
    value = dof * 5 * args.steps / el
    sample = f"{m.description}, the workload's discretisation ({dof} DOF) per step, {args.steps} RK steps, {el:.2f} s"
    line = {"impl": "reference", "metric": metric_name(args.workload), "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": workload_config(args.elems, args.riemann, args.workload),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "C++ restatement of FLEXI's Fortran path (FLEXI needs Fortran, MPI and HDF5, absent here)"}
    print(json.dumps(line), flush=True)


def run_gb300(args):
    import ctypes

    import numpy as np
    import torch

    ws, rank, local = dist_info()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from flexi_gb300 import mesh as fmesh, testcases
    from flexi_gb300.solver import Flexi, probe_fp64_lanes, probe_fp64_pipe, probe_fp64_tensor

    n = args.elems
    kind = args.workload
    cfgd = workload_config(n, args.riemann, kind)
    c = solver_config(args.riemann, kind)
    m = workload_mesh(kind, n, seed=rank)
    f = Flexi(c, m)
    U0 = testcases.tgv_state(f.elem_xgp(), mach=0.1, kappa=1.4, R=71.42857)
    f.U = U0
    f.overintegrate_state()  # timedisc.f90:115-123 (no-op without overintegration)
    dof = f.n_elems * f.n ** 3
    stream = torch.cuda.ExternalStream(f.stream())
    pipe_rates = probe_fp64_pipe()
    tensor_rates = probe_fp64_tensor()
    lane_ms = probe_fp64_lanes()

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()

    # warm-up (graph capture happens here)
    f.TimeDisc(args.warmup)
    # timed region: K steps, per-kernel events on the solver stream
    f.profile(True)
    f.profile_read()
    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    torch.cuda.nvtx.range_push("timed")  # lets a profiler select the timed launches (ncu --nvtx --nvtx-include "timed/")
    f.TimeDisc(args.steps)
    torch.cuda.nvtx.range_pop()
    e1.record(stream)
    barrier()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1)
    prof = f.profile_read()
    launches_per_step = f.launch_count()
    f.profile(False)
    if ws > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    value = dof * 5 * args.steps * ws / (ms * 1e-3)

    # e2e through the public API, state in pinned host memory
    e2e = None
    if not args.no_e2e:
        nbytes = dof * 5 * 8
        hin = torch.empty(dof * 5, dtype=torch.float64).pin_memory()
        hout = torch.empty(dof * 5, dtype=torch.float64).pin_memory()
        f.get_state_ptr(hin.data_ptr())

        def e2e_loop(overlap):
            # upload, step (with the download when overlapped), download; each call returns after its work has finished
            nonlocal hin, hout
            phase = [0.0, 0.0, 0.0]
            barrier()
            t0 = time.perf_counter()
            for _ in range(args.steps):
                ta = time.perf_counter()
                f.set_state_ptr(hin.data_ptr())
                tb = time.perf_counter()
                if overlap:
                    f.TimeDisc_to_host_ptr(1, hout.data_ptr())
                    tc = td = time.perf_counter()
                else:
                    f.TimeDisc(1)
                    tc = time.perf_counter()
                    f.get_state_ptr(hout.data_ptr())
                    td = time.perf_counter()
                phase[0] += tb - ta
                phase[1] += tc - tb
                phase[2] += td - tc
                hin, hout = hout, hin
            barrier()
            el = time.perf_counter() - t0
            if ws > 1:
                t = torch.tensor([el], device="cuda")
                torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
                el = float(t.item())
            return el, [round(x / args.steps * 1e3, 3) for x in phase]

        el, ph = e2e_loop(True)
        el_seq, ph_seq = e2e_loop(False)
        e2e = {"value": dof * 5 * args.steps * ws / el, "unit": UNIT, "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
               "ms_per_step": el / args.steps * 1e3, "ms_per_step_upload_step": ph[:2],
               "api": "fg_set_state, fg_run_to_host (the download overlaps the last stage's volume kernel)",
               "sequential": {"value": dof * 5 * args.steps * ws / el_seq, "ms_per_step": el_seq / args.steps * 1e3,
                              "ms_per_step_upload_step_download": ph_seq, "api": "fg_set_state, fg_run, fg_get_state"}}

    if rank != 0:
        f.close()
        return
    # roofline of the dominant kernel class: bound by FP64 instruction issue (DRAM runs at 5-12 % of its peak)
    dom = max(("prep", "lift", "flux", "vol"), key=lambda k: prof[k][0])
    dom_ms, dom_cnt = prof[dom]
    avg_ms = dom_ms / max(dom_cnt, 1)
    flops = flops_per_dof_stage(args.riemann, kind)
    peaks = measured_peaks()
    hbm_peak = peaks.get("hbm_gbs")
    traffic = ncu_traffic(kind).get(dom)
    instr = fp64_instr(kind).get(dom)
    props = torch.cuda.get_device_properties(local)
    sm_hz = (clk.get("sm_mhz") or 2070.0) * 1e6
    rf = fp64_roofline(instr, dof, avg_ms * 1e-3, props.multi_processor_count, sm_hz, pipe_rates) if instr else {}
    roofline = {"bound": "fp64", "kernel": kernel_names(kind)[dom], "achieved": rf.get("achieved"), "peak": rf.get("peak"),
                "unit": "TFLOP/s", "frac": rf.get("frac"),
                "definition": "executed FP64 flops (DADD, DMUL 1, DFMA 2; ncu counts per DOF x DOF) per launch / CUDA-event launch "
                              "time, against the FP64 pipe's nominal rate for the same instruction mix (2 thread-instructions per "
                              "clock per SM at the SM clock sampled during the timed region; the 100 % of ncu's "
                              "sm__pipe_fp64_cycles_active)",
                "attainable": "a stream of DFMA, DADD or DMUL alone or mixed, any launch shape, attains %.4f of the nominal rate "
                              "(fg_probe_fp64_pipe on this GPU: T instr/s DFMA %.4f, DADD %.4f, DMUL %.4f, mixed %.4f)"
                              % (rf.get("attainable_frac_of_nominal") or float("nan"), pipe_rates["dfma"], pipe_rates["dadd"], pipe_rates["dmul"],
                                 pipe_rates["mixed"]),
                "frac_of_attainable": rf.get("frac_of_attainable"), "sm_clock_hz": sm_hz, "sms": props.multi_processor_count,
                "fp64_tensor_tflops": dict(tensor_rates, note="mma.sync m8n8k4 f64 alone, and interleaved with DFMA (both "
                                           "counted): not above the DFMA pipe's own rate, the FP64 tensor path shares the FP64 units"),
                "fp64_idle_lanes_ms": dict(lane_ms, note="the same DFMA chains with 32/16/8/4/1 active lanes per warp: equal "
                                           "times, so idle lanes of FP64 code cost pipe time like active ones"),
                "fp64_instr_per_dof": instr, "ncu_fp64_pipe_active_pct": instr.get("pipe_active_pct") if instr else None,
                "traffic": (traffic * dof if traffic is not None else None),
                "traffic_unit": "bytes per launch (ncu dram read+write, scaled per DOF)" if traffic is not None else None,
                "algorithmic_flops_per_dof": flops[dom], "algorithmic_tflops": flops[dom] * dof / (avg_ms * 1e-3) / 1e12,
                "avg_launch_ms": avg_ms,
                "hbm_alg_gbs": value / ws * BYTES_ALG_PER_DOF_STAGE / 1e9,
                "hbm_peak_gbs": hbm_peak or HBM_FALLBACK_GBS,
                "hbm_peak_source": "MEASURED_PEAKS.json" if hbm_peak else "fallback (no MEASURED_PEAKS.json on this box)",
                "frac_hbm": value / ws * BYTES_ALG_PER_DOF_STAGE / 1e9 / (hbm_peak or HBM_FALLBACK_GBS),
                "kernel_ms_per_step": {k: prof[k][0] / args.steps for k in prof}}
    try:
        if args.no_cpu_baseline:
            raise RuntimeError("skipped (--no-cpu-baseline)")
        cpu_val, cores, sample = cpu_baseline_sample(args.riemann, kind=kind)
        cpu = {"value": cpu_val, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample}
    except Exception as ex:  # reported, never substituted for the GPU path
        cpu = {"value": None, "unit": UNIT, "cores": None, "kind": "port", "sample": f"failed: {ex}"}
    line = {"metric": metric_name(kind), "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": cfgd, "e2e": e2e, "gpu_launches": launches_per_step * args.steps, "clocks": clk,
            "roofline": roofline, "cpu_baseline": cpu}
    f.close()
    if args.riemann == "hllc" and kind == "tgv":
        # the same workload with the surface flux of the reference's split-form TGV regression (the parity setting)
        c2 = solver_config("roeentropyfix")
        g = Flexi(c2, m)
        g.U = U0
        g.TimeDisc(args.warmup)
        gs = torch.cuda.ExternalStream(g.stream())
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(gs)
        g.TimeDisc(args.steps)
        b.record(gs)
        torch.cuda.synchronize()
        ms2 = a.elapsed_time(b)
        line["variant_roeentropyfix"] = {"value": dof * 5 * args.steps / (ms2 * 1e-3), "unit": UNIT, "ms_per_step": ms2 / args.steps,
                                         "workload": workload_config(n, "roeentropyfix")["workload"]}
        g.close()
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------------------------------------
# Ensemble workload: independent periodic instances of uneven size and flow parameters in one solver
# ---------------------------------------------------------------------------------------------------------
ENSEMBLE_SIZES = (4, 6, 8, 12, 16)
# The ensemble's discretisation is the split form PI on Gauss nodes (N=5, RoeEntropyFix, BR1; the reference's
# tgv/splitGauss setting): over its 500 steps the weak form lets an under-resolved instance (4^3 elements, TGV at
# Re 2119, Ma 0.28) diverge near t = 4.9, the split form keeps every instance bounded. Oracle flop counts per DOF and
# stage are those of that discretisation.
ENSEMBLE_FLOPS = dict(SPLITGAUSS_FLOPS_PER_DOF_STAGE)
ENSEMBLE_METRIC = "ensemble instance-steps/s (256 TGV/vortex instances, N=5 Gauss)"


def ensemble_spec(n_inst, seed=0):
    """Seeded instance parameters: elements per direction, Mach number U[0.05,0.3], Reynolds number
    logU[400,3200], kind (0 Taylor-Green vortex, 1 isentropic vortex)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    sizes = rng.choice(ENSEMBLE_SIZES, size=n_inst)
    mach = rng.uniform(0.05, 0.3, n_inst)
    re = np.exp(rng.uniform(np.log(400.0), np.log(3200.0), n_inst))
    kind = rng.integers(0, 2, n_inst)
    return sizes, mach, re, kind


def ensemble_solver_config():
    from flexi_gb300.solver import make_config
    return make_config(N=5, NodeType="gauss", SplitDG="pi", Riemann="roeentropyfix", Lifting="br1", kappa=1.4, R=71.42857, Pr=0.72,
                       mu0=1.0 / 1600.0, CFLScale=0.9, DFLScale=0.9)


def ensemble_oracle_config():
    return dict(N=5, nodeType=1, riemann=33, riemannBC=-1, lifting=1, weakLifting=0, consLifting=0, splitDG=4, etaBR2=2.0, etaBR2_wall=-1.0,
                kappa=1.4, R=71.42857, Pr=0.72, mu0=1.0 / 1600.0, CFLScale=0.9, DFLScale=0.9, doTCSource=0, dpdx=-1.0)


def instance_state(xgp, kind, mach):
    from flexi_gb300 import testcases
    if kind == 0:
        return testcases.tgv_state(xgp, mach=mach, kappa=1.4, R=71.42857)
    return testcases.shu_vortex_state(xgp, mach=mach, kappa=1.4)


def ensemble_config(sizes, n_dof):
    return {"workload": f"ensemble of {len(sizes)} periodic TGV / isentropic-vortex instances, elements per instance drawn from "
                        f"{{4,6,8,12,16}}^3, Ma U[0.05,0.3], Re logU[400,3200] (seeded), N=5 Gauss, split form PI, RoeEntropyFix, BR1, FP64",
            "instances": len(sizes), "n_elems": int(sum(int(k) ** 3 for k in sizes)), "N": 5, "dof": n_dof, "CFLScale": 0.9, "DFLScale": 0.9,
            "time_integration": "CarpenterRK4-5, per-instance CFL/DFL dt each step, one graph-replayed launch sequence for all instances, "
                                "launch shapes autotuned (fg_autotune); the per-instance loop uses the default shapes",
            "l2": f"inputs larger than L2 (state {n_dof * 40 / 1e9:.1f} GB)", "parallelism": "replicas"}


def run_ensemble(args):
    import numpy as np
    import torch

    ws, rank, local = dist_info()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from flexi_gb300 import mesh as fmesh
    from flexi_gb300.solver import Flexi, probe_fp64_pipe

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()

    sizes, mach, re, kind = ensemble_spec(args.instances, seed=rank)
    c = ensemble_solver_config()
    boxes = {int(k): fmesh.tgv_box(int(k)) for k in set(sizes.tolist())}
    m = fmesh.concatenate([boxes[int(k)] for k in sizes])
    f = Flexi(c, m)
    xgp = f.elem_xgp()
    starts = np.concatenate([[0], np.cumsum(sizes.astype(np.int64) ** 3)])
    f_n3 = (c.N + 1) ** 3
    U0 = np.concatenate([instance_state(xgp[starts[i]:starts[i + 1]], int(kind[i]), float(mach[i])) for i in range(len(sizes))])
    mu = 1.0 / re
    f.U = U0
    f.set_instance_mu0(mu)
    dof = f.n_elems * f.n ** 3
    stream = torch.cuda.ExternalStream(f.stream())
    pipe_rates = probe_fp64_pipe()
    # launch shapes of the ensemble's kernels picked by timing the candidates on this mesh and state
    tuned = f.autotune(reps=5)

    f.TimeDisc(args.warmup)
    f.profile(True)
    f.profile_read()
    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    torch.cuda.nvtx.range_push("timed")  # lets a profiler select the timed launches (ncu --nvtx --nvtx-include "timed/")
    f.TimeDisc(args.steps)
    torch.cuda.nvtx.range_pop()
    e1.record(stream)
    barrier()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1)
    prof = f.profile_read()
    launches_per_step = f.launch_count()
    f.profile(False)
    U_ens = f.U
    if ws > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    value = len(sizes) * args.steps * ws / (ms * 1e-3)

    # e2e through the public API: host state in, one step for all instances, host state out (a sample of at most 50
    # steps from the initial state: the rate does not depend on the step count)
    e2e = None
    if not args.no_e2e:
        f.U = U0
        nbytes = dof * 5 * 8
        n_e2e = min(args.steps, 50)
        hin = torch.from_numpy(np.ascontiguousarray(U0).reshape(-1)).pin_memory()
        hout = torch.empty(dof * 5, dtype=torch.float64).pin_memory()
        barrier()
        t0 = time.perf_counter()
        for _ in range(n_e2e):
            f.set_state_ptr(hin.data_ptr())
            f.TimeDisc_to_host_ptr(1, hout.data_ptr())
            hin, hout = hout, hin
        barrier()
        el = time.perf_counter() - t0
        e2e = {"value": len(sizes) * n_e2e * ws / el, "unit": "instance-steps/s", "h2d_bytes_per_step": nbytes,
               "d2h_bytes_per_step": nbytes, "ms_per_step": el / n_e2e * 1e3, "steps": n_e2e,
               "api": "fg_set_state, fg_run_to_host (the download overlaps the last stage)"}
    f.close()

    # the same instances, one plain solver after another (same kernels, same steps, graph-replayed per instance),
    # with the time per instance size
    loop_ms, max_diff = 0.0, 0.0
    per_size = {}
    for i in range(len(sizes)):
        g = Flexi(c, boxes[int(sizes[i])])
        g.U = U0[starts[i]:starts[i + 1]]
        g.set_instance_mu0(np.array([mu[i]]))
        g.TimeDisc(args.warmup)
        gs = torch.cuda.ExternalStream(g.stream())
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(gs)
        g.TimeDisc(args.steps)
        b.record(gs)
        torch.cuda.synchronize()
        ms_i = a.elapsed_time(b)
        loop_ms += ms_i
        ps = per_size.setdefault(int(sizes[i]), {"instances": 0, "ms": 0.0, "dof": 0})
        ps["instances"] += 1
        ps["ms"] += ms_i
        ps["dof"] += int(sizes[i]) ** 3 * f_n3
        ref = U_ens[starts[i]:starts[i + 1]]
        max_diff = max(max_diff, float(np.abs(g.U - ref).max() / np.abs(ref).max()))
        g.close()
    loop_value = len(sizes) * args.steps / (loop_ms * 1e-3)
    ens_rate = dof * 5 * args.steps / (ms * 1e-3)
    # per instance size: share of the loop's time and of the DOF, DOF*stage/s of an instance of that size run alone
    # against the ensemble's rate (instances too small to fill the GPU run below it)
    loop_breakdown = {f"{k}^3": {"instances": v["instances"], "elements": k ** 3, "dof_share": v["dof"] / dof,
                                  "loop_time_share": v["ms"] / loop_ms,
                                  "ms_per_step_all_instances": v["ms"] / args.steps,
                                  "dof_stage_per_s_alone": v["dof"] * 5 * args.steps / (v["ms"] * 1e-3),
                                  "rate_vs_ensemble": v["dof"] * 5 * args.steps / (v["ms"] * 1e-3) / ens_rate}
                      for k, v in sorted(per_size.items())}
    # Amdahl bound of batching: the ensemble cannot beat the loop by more than running every size class at the rate of
    # the best-filled one
    best = max(v["dof_stage_per_s_alone"] for v in loop_breakdown.values())
    amdahl = loop_ms * 1e-3 / sum(v["dof"] * 5 * args.steps / best for v in per_size.values())

    if rank != 0:
        return
    dom = max(("prep", "lift", "flux", "vol"), key=lambda k: prof[k][0])
    avg_ms = prof[dom][0] / max(prof[dom][1], 1)
    instr = fp64_instr("ensemble").get(dom)
    props = torch.cuda.get_device_properties(local)
    sm_hz = (clk.get("sm_mhz") or 2070.0) * 1e6
    rf = fp64_roofline(instr, dof, avg_ms * 1e-3, props.multi_processor_count, sm_hz, pipe_rates) if instr else {}
    roofline = {"bound": "fp64", "kernel": {"vol": "k_vol_split_gen<6,Gauss>", "lift": "k_lift<6,Gauss>", "flux": "k_flux<6>", "prep": "k_prep<6,Gauss>"}[dom],
                "achieved": rf.get("achieved"), "peak": rf.get("peak"), "unit": "TFLOP/s", "frac": rf.get("frac"),
                "definition": "executed FP64 flops per launch / launch time against the FP64 pipe's nominal rate for the same "
                              "instruction mix (2 thread-instructions per clock per SM)",
                "frac_of_attainable": rf.get("frac_of_attainable"), "attainable_frac_of_nominal": rf.get("attainable_frac_of_nominal"),
                "fp64_instr_per_dof": instr, "traffic": None,
                "algorithmic_flops_per_dof": ENSEMBLE_FLOPS[dom], "algorithmic_tflops": ENSEMBLE_FLOPS[dom] * dof / (avg_ms * 1e-3) / 1e12,
                "avg_launch_ms": avg_ms, "kernel_ms_per_step": {k: prof[k][0] / args.steps for k in prof}}
    try:
        if args.no_cpu_baseline:
            raise RuntimeError("skipped (--no-cpu-baseline)")
        cpu = ensemble_cpu_baseline()
    except Exception as ex:
        cpu = {"value": None, "unit": "instance-steps/s", "cores": None, "kind": "port", "sample": f"failed: {ex}"}
    line = {"metric": ENSEMBLE_METRIC, "value": value, "unit": "instance-steps/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic", "config": ensemble_config(sizes, dof), "e2e": e2e,
            "gpu_launches": launches_per_step * args.steps, "clocks": clk, "roofline": roofline, "cpu_baseline": cpu,
            "dof_stage_per_s": dof * 5 * args.steps * ws / (ms * 1e-3),
            "loop_baseline": {"value": loop_value, "unit": "instance-steps/s", "ms_per_step": loop_ms / args.steps,
                              "what": "the same instances advanced one after another by the plain solver (one handle per instance)",
                              "per_instance_size": loop_breakdown,
                              "batching_bound": amdahl,
                              "batching_bound_note": "largest speed-up over the loop that batching can give: every size class "
                                                     "run at the DOF*stage/s of the best-filled size alone"},
            "speedup_vs_loop": value / ws / loop_value, "max_rel_state_diff_vs_loop": max_diff,
            "autotune": tuned}
    print(json.dumps(line), flush=True)


def ensemble_cpu_baseline(budget_s=10.0):
    """Oracle on all host threads, instance by instance over the first instances of the ensemble."""
    import numpy as np
    from flexi_gb300 import mesh as fmesh
    from oracle import oracle as orc
    orc.set_threads(os.cpu_count() or 1)
    sizes, mach, re, kind = ensemble_spec(8)
    done, el = 0, 0.0
    for i in range(len(sizes)):
        cfg = dict(ensemble_oracle_config(), mu0=float(1.0 / re[i]))
        m = fmesh.tgv_box(int(sizes[i]))
        o = orc.Oracle(cfg, m)
        o.set_state(instance_state(o.mesh_array("Elem_xGP"), int(kind[i]), float(mach[i])))
        t = 0.0
        t0 = time.perf_counter()
        for _ in range(2):
            dt, _ = o.calc_timestep()
            t = o.timestep(t, dt)
            done += 1
        el += time.perf_counter() - t0
        if el > budget_s:
            break
    return {"value": done / el, "unit": "instance-steps/s", "cores": orc.max_threads(), "kind": "port",
            "sample": f"first {i + 1} instances of the same seeded ensemble (sizes {sizes[:i + 1].tolist()}), 2 RK steps each, "
                      f"{el:.1f} s of stepping"}


# ---------------------------------------------------------------------------------------------------------
# Differentiation workload: adjoint of a checkpointed fixed-dt solve
# ---------------------------------------------------------------------------------------------------------
ADJOINT_METRIC = "adjoint/forward cost ratio (TGV 16^3, N=5 Gauss, 200 LSERK steps)"
ORACLE_ADJ_CFG = dict(N=5, nodeType=1, riemann=33, riemannBC=-1, lifting=1, weakLifting=0, consLifting=0, splitDG=-1, etaBR2=2.0, etaBR2_wall=-1.0,
                      kappa=1.4, R=71.42857, Pr=0.72, mu0=1.0 / 1600.0, CFLScale=0.9, DFLScale=0.9, doTCSource=0, dpdx=-1.0)


def run_adjoint(args):
    import numpy as np
    import torch

    ws, rank, local = dist_info()
    torch.cuda.set_device(local)
    from flexi_gb300 import mesh as fmesh, testcases
    from flexi_gb300.solver import Flexi, make_config
    from oracle import oracle as orc

    n_el, n_steps = 16, 200 if args.steps == 20 else args.steps
    c = make_config(N=5, NodeType="gauss", SplitDG="weak", Riemann="roeentropyfix", Lifting="br1", kappa=1.4, R=71.42857, Pr=0.72,
                    mu0=1.0 / 1600.0, CFLScale=0.9, DFLScale=0.9)
    m = fmesh.tgv_box(n_el)
    f = Flexi(c, m)
    rng = np.random.default_rng(1234 + rank)
    U0 = testcases.tgv_state(f.elem_xgp(), mach=0.1, kappa=1.4, R=71.42857)
    scale = rng.uniform(0.8, 1.2, f.n_elems)
    f.U = U0
    f.set_elem_mu_scale(scale)
    dt = float(np.atleast_1d(f.CalcTimeStep()[0])[0])
    dof = f.n_elems * f.n ** 3
    _, w1, _ = orc.nodes_and_weights(5, 1)
    wq = np.einsum("k,j,i->kji", w1, w1, w1)[None] / f.mesh_array("sJ")  # quadrature weight x Jacobian

    def kinetic_terms(U):
        return 0.5 * (U[..., 1] ** 2 + U[..., 2] ** 2 + U[..., 3] ** 2) / U[..., 0] * wq

    def kinetic(U):
        return float(kinetic_terms(U).sum())

    target = kinetic(U0) * rng.uniform(0.9, 0.95)

    def final_state(U0_, s_):
        # the same fixed-dt solve through the reference-facing step entry (TimeStepByLSERKW2)
        f.U = U0_
        f.set_elem_mu_scale(s_)
        t = 0.0
        for _ in range(n_steps):
            t = f.TimeStepByLSERKW2(t, dt)
        return f.U

    def loss_difference(Up, Um):
        # L(Up) - L(Um) = 1/2 (K+ - K-) (K+ + K- - 2 target), with K+ - K- summed from the nodes' differences: two
        # separately rounded sums K+ and K- would leave about 1e-16 K of round-off in their difference
        kp, km = kinetic_terms(Up), kinetic_terms(Um)
        return 0.5 * float((kp - km).sum()) * (float(kp.sum()) + float(km.sum()) - 2.0 * target)

    stream = torch.cuda.ExternalStream(f.stream())

    def timed(fn):
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        out = fn()
        b.record(stream)
        torch.cuda.synchronize()
        return out, a.elapsed_time(b)

    # warm-up (kernel loading, buffer allocation); the adjoint's device footprint is measured against the
    # free memory before it
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    f.U = U0
    f.adjoint_forward(args.warmup, dt, args.ckpt)
    f.adjoint_reverse(np.zeros(f.ushape))
    # plain forward: the solver's own time loop (graph-replayed, dt from CALCTIMESTEP each step)
    f.U = U0
    f.set_elem_mu_scale(scale)
    f.TimeDisc(2)
    f.U = U0
    _, ms_plain = timed(lambda: f.TimeDisc(n_steps))
    plain_launches = f.launch_count() * n_steps  # per step of the captured loop
    # forward with checkpoints, then the reverse sweep
    f.U = U0
    clocks = ClockSampler(local)
    clocks.start()
    _, ms_fwd = timed(lambda: f.adjoint_forward(n_steps, dt, args.ckpt))
    fwd_launches = f.launch_count()
    adj_bytes = free0 - torch.cuda.mem_get_info()[0]
    UT = f.U
    KE = kinetic(UT)
    UbarT = np.zeros(f.ushape)
    rho = UT[..., 0]
    UbarT[..., 0] = -0.5 * (UT[..., 1] ** 2 + UT[..., 2] ** 2 + UT[..., 3] ** 2) / rho ** 2 * wq
    for c_ in (1, 2, 3):
        UbarT[..., c_] = UT[..., c_] / rho * wq
    UbarT *= KE - target
    (Ub0, mub), ms_rev = timed(lambda: f.adjoint_reverse(UbarT))
    rev_launches = f.launch_count()
    clk = clocks.stop()
    L0 = 0.5 * (KE - target) ** 2
    # finite differences of the loss in seeded random directions of (U0, multipliers): the central difference with
    # eps = 1e-6, and central differences at h, 2h, 4h (h = 2e-5) extrapolated twice (Richardson: fourth order from h, 2h,
    # sixth order from all three). Each quotient differences the two final states node by node before summing
    # (loss_difference). The distance between the fourth- and sixth-order values estimates the fourth-order one's
    # truncation error, and that of the eps = 1e-6 quotient from the sixth-order value is that quotient's own error; the
    # exact tangent (--exact-dirs) measures both FD values' errors.
    errs, errs_rich, fd_own, rich_own, exact = [], [], [], [], []
    o_ex = None
    h = 2e-5
    for k in range(args.fd_dirs):
        dU = rng.standard_normal(U0.shape) * np.abs(U0).max(axis=(0, 1, 2, 3))
        ds = rng.standard_normal(f.n_elems)
        eps = 1e-6
        fd = loss_difference(final_state(U0 + eps * dU, scale + eps * ds), final_state(U0 - eps * dU, scale - eps * ds)) / (2 * eps)
        D = [loss_difference(final_state(U0 + k_ * h * dU, scale + k_ * h * ds), final_state(U0 - k_ * h * dU, scale - k_ * h * ds)) /
             (2 * k_ * h) for k_ in (1, 2, 4)]
        r4 = [(4 * D[0] - D[1]) / 3, (4 * D[1] - D[2]) / 3]
        rich = (16 * r4[0] - r4[1]) / 15
        ad = float((Ub0 * dU).sum() + mub @ ds)
        den = max(abs(rich), 1e-300)
        errs.append(abs(ad - fd) / max(abs(fd), 1e-300))
        errs_rich.append(abs(ad - rich) / den)
        fd_own.append(abs(fd - rich) / den)
        rich_own.append(abs(r4[0] - rich) / den)
        if k < args.exact_dirs:
            # the exact tangent of the oracle's own solve of the same steps along the same direction (dual numbers):
            # the FD quotients' error against it, and the adjoint's
            if o_ex is None:
                orc.set_threads(os.cpu_count() or 1)
                o_ex = orc.Oracle(ORACLE_ADJ_CFG, m)
            o_ex.set_state(U0)
            o_ex.set_mu_scale(scale)
            t0 = time.perf_counter()
            JV = o_ex.jvp_solve(dU, n_steps, dt, d_scale=ds)
            ex = float((UbarT * JV).sum())
            exact.append({"direction": k, "adjoint_vs_exact": abs(ad - ex) / abs(ex), "richardson_vs_exact": abs(rich - ex) / abs(ex),
                          "eps_1e-6_vs_exact": abs(fd - ex) / abs(ex), "oracle_s": time.perf_counter() - t0})
    # dot-product test at t_end against the reference's matrix-free FD JVP (FD_Order 2) on the oracle
    o = orc.Oracle(ORACLE_ADJ_CFG, m)
    o.set_state(UT)
    o.set_mu_scale(scale)
    V = rng.standard_normal(UT.shape) * np.abs(UT).max(axis=(0, 1, 2, 3))
    W = rng.standard_normal(UT.shape)
    JV = o.fd_jvp(V, fd_order=2, eps_method=1)
    f.U = UT
    f.set_elem_mu_scale(scale)
    JTW, _ = f.vjp_time_derivative(W)
    dot_err = abs(float((JV * W).sum()) - float((V * JTW).sum())) / float(np.abs(JV * W).sum())
    nck = (n_steps + args.ckpt - 1) // args.ckpt
    mem_states_gb = (nck + 5 * args.ckpt + 3) * dof * 5 * 8 / 1e9
    if rank != 0:
        return
    line = {"metric": ADJOINT_METRIC, "value": ms_rev / ms_plain, "unit": "reverse time / forward time", "n_gpus": ws,
            "steps": n_steps, "warmup": args.warmup, "ms_per_step": ms_rev / n_steps, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"TGV {n_el}^3 Cartesian, N=5 Gauss, weak form, RoeEntropyFix, BR1, Re=1600, Ma=0.1, FP64, {n_steps} "
                                   f"LSERK steps of fixed dt, checkpoint every {args.ckpt} steps; loss 1/2 (KE(t_end) - target)^2; "
                                   "gradient w.r.t. U0 and per-element viscosity multipliers U[0.8,1.2]",
                       "n_elems": f.n_elems, "N": 5, "dof": dof, "dt": dt, "l2": "inputs larger than L2 (state 35 MB, stage states 3.5 GB)"},
            "forward_ms_per_step": ms_plain / n_steps, "forward": "the plain solver's graph-replayed time loop (fg_run)",
            "forward_with_checkpoints_ms_per_step": ms_fwd / n_steps,
            "reverse_ms_per_step": ms_rev / n_steps,
            "reverse_includes": "recomputation of every segment's stage states from its checkpoint + 5 adjoint right-hand sides per step",
            "adjoint_device_memory_gb": adj_bytes / 1e9, "checkpoint_and_stage_states_gb": mem_states_gb,
            "stage_intermediates_kept": adj_bytes / 1e9 > 1.5 * mem_states_gb, "loss": L0,
            "fd_check": {"directions": args.fd_dirs, "eps": 1e-6, "max_rel_err": max(errs) if errs else None,
                         "median_rel_err": float(np.median(errs)) if errs else None,
                         "richardson_h": h, "richardson_order": 6, "max_rel_err_vs_richardson": max(errs_rich) if errs_rich else None,
                         "median_rel_err_vs_richardson": float(np.median(errs_rich)) if errs_rich else None,
                         "eps_1e-6_quotient_own_error_max": max(fd_own) if fd_own else None,
                         "richardson_4th_order_own_error_max": max(rich_own) if rich_own else None,
                         "exact_tangent": exact,
                         "adjoint_vs_exact_max": max((x["adjoint_vs_exact"] for x in exact), default=None),
                         "richardson_vs_exact_max": max((x["richardson_vs_exact"] for x in exact), default=None),
                         "note": "central FD at eps=1e-6 as the configuration states, and central FDs at h=2e-5, 2h, 4h extrapolated to "
                                 "sixth order; each quotient sums the node-by-node differences of the two final states' kinetic "
                                 "energies; the sixth-order value's distance from the eps=1e-6 quotient is that quotient's own error, "
                                 "its distance from the fourth-order value (h, 2h) bounds the fourth-order value's"},
            "dot_product_vs_reference_fd_jvp": {"rel_err": dot_err, "fd": "implicit.f90:MatrixVector FD_Order 2, Eps_Method 1, on the oracle"},
            "e2e": {"value": ms_rev / ms_plain, "unit": "reverse time / forward time", "h2d_bytes_per_step": dof * 5 * 8 / n_steps,
                    "d2h_bytes_per_step": (dof * 5 * 8 + f.n_elems * 8) / n_steps},
            "gpu_launches": rev_launches, "gpu_launches_forward_checkpointed": fwd_launches, "gpu_launches_forward_plain": plain_launches,
            "clocks": clk}
    print(json.dumps(line), flush=True)


ADJOINT_CHANNEL_METRIC = "adjoint/forward cost ratio (channel 24x12x12, N=7 GL split PI, 500 LSERK steps)"


def run_adjoint_channel(args):
    """Gradient of the mean wall shear after a forward channel solve with respect to the body-force field."""
    import numpy as np
    import torch

    ws, rank, local = dist_info()
    torch.cuda.set_device(local)
    from flexi_gb300 import mesh as fmesh, testcases
    from flexi_gb300.solver import Flexi, make_config

    n_steps = 500 if args.steps == 20 else args.steps
    mu0 = 1.0 / 2800.0  # Re_b = rho_b U_b h / mu = 2800 with rho_b = U_b = h = 1
    dpdx = -3.0 * mu0   # the body force that balances the wall shear of the laminar profile
    c = make_config(N=7, NodeType="gauss-lobatto", SplitDG="pi", Riemann="roe", Lifting="br1", kappa=1.4, R=1.0, Pr=0.72, mu0=mu0,
                    CFLScale=0.8, DFLScale=0.8, doTCSource=1, dpdx=dpdx)
    m = fmesh.channel_box((24, 12, 12), beta=1.5, t_wall=1.0)
    f = Flexi(c, m)
    xgp = f.elem_xgp()
    U0 = testcases.channel_state(xgp, mach=0.1, kappa=1.4, R=1.0, t_wall=1.0, noise=0.05, seed=rank)
    f.U = U0
    dt = float(np.atleast_1d(f.CalcTimeStep()[0])[0])
    dof = f.n_elems * f.n ** 3
    stream = torch.cuda.ExternalStream(f.stream())

    def timed(fn):
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        out = fn()
        b.record(stream)
        torch.cuda.synchronize()
        return out, a.elapsed_time(b)

    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    f.adjoint_forward(args.warmup, dt, args.ckpt)
    f.adjoint_reverse(np.zeros(f.ushape))
    f.U = U0
    f.TimeDisc(2)
    f.U = U0
    _, ms_plain = timed(lambda: f.TimeDisc(n_steps))
    plain_launches = f.launch_count() * n_steps
    f.U = U0
    clocks = ClockSampler(local)
    clocks.start()
    _, ms_fwd = timed(lambda: f.adjoint_forward(n_steps, dt, args.ckpt))
    fwd_launches = f.launch_count()
    adj_bytes = free0 - torch.cuda.mem_get_info()[0]
    (J, dJdU), ms_seed = timed(lambda: f.wall_shear(grad=True))
    (Ub0, mub, Fbar), ms_rev = timed(lambda: f.adjoint_reverse(dJdU, force_bar=True))
    rev_launches = f.launch_count()
    clk = clocks.stop()
    # directional check along one smooth body-force mode with a Richardson-extrapolated central difference
    # of the same fixed-dt solve (approximate: the Roe flux has kinks a difference quotient can straddle)
    dF = 0.1 * abs(dpdx) * np.cos(xgp[..., 0]) * (1.0 - xgp[..., 1] ** 2)

    def J_of(h):
        f.set_body_force_field(h * dF)
        f.U = U0
        t = 0.0
        for _ in range(n_steps):
            t = f.TimeStepByLSERKW2(t, dt)
        return f.wall_shear()

    d1 = (J_of(1.0) - J_of(-1.0)) / 2.0
    d2 = (J_of(2.0) - J_of(-2.0)) / 4.0
    f.set_body_force_field(None)
    fd = (4.0 * d1 - d2) / 3.0
    ad = float((Fbar * dF).sum())
    if rank != 0:
        return
    line = {"metric": ADJOINT_CHANNEL_METRIC, "value": ms_rev / ms_plain, "unit": "reverse time / forward time", "n_gpus": ws,
            "steps": n_steps, "warmup": args.warmup, "ms_per_step": ms_rev / n_steps, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"channel [0,2pi]x[-1,1]x[0,pi], 24x12x12 elements tanh-stretched (beta=1.5), isothermal walls, "
                                   f"N=7 Gauss-Lobatto, split PI, Roe, BR1, body force dpdx=-3 mu, Ma=0.1, Re_b=2800, laminar profile + 5% "
                                   f"seeded noise, FP64, {n_steps} LSERK steps of fixed dt, checkpoint every {args.ckpt} steps; gradient of the "
                                   "mean wall shear at t_end w.r.t. the body-force field",
                       "n_elems": f.n_elems, "N": 7, "dof": dof, "dt": dt, "l2": "inputs larger than L2 (state 71 MB)"},
            "forward_ms_per_step": ms_plain / n_steps, "forward": "the plain solver's graph-replayed time loop (fg_run)",
            "forward_with_checkpoints_ms_per_step": ms_fwd / n_steps, "reverse_ms_per_step": ms_rev / n_steps,
            "wall_shear_gradient_ms": ms_seed, "adjoint_device_memory_gb": adj_bytes / 1e9, "mean_wall_shear": J,
            "body_force_gradient_norm": float(np.sqrt((Fbar ** 2).sum())),
            "fd_check": {"direction": "0.1 |dpdx| cos(x) (1 - y^2)", "adjoint": ad, "fd_richardson": fd,
                         "rel_err": abs(ad - fd) / max(abs(fd), 1e-300)},
            "e2e": {"value": ms_rev / ms_plain, "unit": "reverse time / forward time", "h2d_bytes_per_step": dof * 5 * 8 / n_steps,
                    "d2h_bytes_per_step": dof * 6 * 8 / n_steps},
            "gpu_launches": rev_launches, "gpu_launches_forward_checkpointed": fwd_launches, "gpu_launches_forward_plain": plain_launches,
            "clocks": clk}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "ensemble":
        run_ensemble(args)
    elif args.workload == "adjoint":
        run_adjoint(args)
    elif args.workload == "adjoint-channel":
        run_adjoint_channel(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
