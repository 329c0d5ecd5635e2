"""Benchmark of the assembly hot path on the 3D variable-coefficient Poisson workload.

Workload: unit cube, 128^3 Q1 hex cells, parts (2,2,2) as 8 slabs on one GPU,
kappa = exp(g) with g a seeded Gaussian random field (sigma 1, squared-exponential
correlation length 0.1) at the cell centres, f = 1, homogeneous Dirichlet,
quadrature degree 2.  A "step" is one numeric assembly of matrix values and
right-hand side into the cached symbolic pattern (assemble_matrix_and_vector!),
SubAssembledRows.

Metric: assembled matrix entries per second (the global matrix's nnz divided by the
step time), whole job.  `e2e` is the same metric through the C-ABI call with host
buffers: kappa copied host->device and the assembled values + rhs copied
device->host inside every timed step.  `roofline` uses the algorithmic bytes
8*nnz + 8*n_free + 8*n_cells per assembly against the measured HBM copy bandwidth.
`solve` reports Jacobi-PCG (FP64) and the mixed-precision refinement to 1e-8 relative
residual on the assembled system; `learned` the learned-preconditioner flexible CG
against both on 96^3 lognormal diffusion (sigma 1.5); `batched` the 64-problem uneven
batch (Q1-Q3, 16^3..96^3 cells) assembled one persistent launch per memory wave; `c1` the
2D Q2 Poisson problem on 128^2 cells (u = (x+y)^2 on the boundary, f = -4): assembly,
solves and the known-answer L2 error.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
Under torchrun with N>1 every rank runs its own replica of the workload on its own
GPU (weak scaling, no data-path collective); the max time over ranks is reported.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
PKG = ROOT / "gridapdistributed.jl_gb300"
sys.path.insert(0, str(PKG))

METRIC = "assembly nnz/s (HBM % of peak); solve s to 1e-8 rel. res., learned vs Jacobi"
UNIT = "nnz/s"
L2_FLUSH_BYTES = 512 << 20   # > 129 MB L2


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-solve", action="store_true")
    ap.add_argument("--solve-maxit", type=int, default=20000)
    ap.add_argument("--cells", type=int, default=128, help="cells per direction (default: the 128^3 workload)")
    ap.add_argument("--batched", default="sample", choices=["off", "sample", "full"],
                    help="batched 64-problem workload: a bounded first wave (sample), every wave (full) or none")
    ap.add_argument("--batched-budget-gb", type=float, default=140.0, help="device memory per wave (full)")
    ap.add_argument("--batched-sample-gb", type=float, default=16.0, help="device memory of the sample wave")
    ap.add_argument("--no-batched-solve", dest="batched_solve", action="store_false",
                    help="skip the batched Jacobi-PCG of every problem of the sample wave")
    ap.add_argument("--no-learned", action="store_true")
    ap.add_argument("--no-c1", action="store_true", help="skip the 2D Q2 128^2 Poisson section")
    ap.add_argument("--no-elasticity", action="store_true")
    ap.add_argument("--no-elasticity-solve", dest="elasticity_solve", action="store_false",
                    help="skip the elasticity solves to 1e-8 (about 30 s)")
    ap.add_argument("--elasticity-cells", type=int, default=64, help="cells per direction of the elasticity workload")
    ap.add_argument("--no-qp", action="store_true", help="skip the Gauss-point elasticity section (tensor cores)")
    ap.add_argument("--qp-cells", type=int, default=64, help="cells per direction of the Gauss-point workload")
    return ap.parse_args()


def gpu_numa_node(local):
    """NUMA node of the host CPUs attached to GPU `local` (its PCI device in sysfs), or None."""
    try:
        bus = subprocess.run(["nvidia-smi", "-i", str(local), "--query-gpu=pci.bus_id", "--format=csv,noheader"],
                             capture_output=True, text=True, timeout=30).stdout.strip()
    except (OSError, subprocess.SubprocessError):
        return None
    if ":" not in bus:
        return None
    dom, rest = bus.split(":", 1)   # nvidia-smi prints an 8-digit PCI domain, sysfs a 4-digit one
    try:
        names = [f"{int(dom, 16):04x}:{rest}".lower(), bus.lower()]
    except ValueError:
        return None
    for name in names:
        f = Path("/sys/bus/pci/devices") / name / "numa_node"
        if f.exists():
            try:
                node = int(f.read_text().strip())
            except ValueError:
                return None
            return node if node >= 0 else None
    return None


def bind_host_to_gpu(local):
    """Run on the CPUs of the GPU's own NUMA node, so that the pinned host buffers of the
    end-to-end measurement (first touched by this thread) sit next to the GPU; returns the
    node, or None where the topology is not visible (nothing changed then)."""
    node = gpu_numa_node(local)
    if node is None:
        return None
    f = Path(f"/sys/devices/system/node/node{node}/cpulist")
    if not f.exists():
        return None
    cpus = set()
    for part in f.read_text().strip().split(","):
        if not part:
            continue
        a, _, b = part.partition("-")
        cpus.update(range(int(a), int(b or a) + 1))
    if not cpus:
        return None
    try:
        os.sched_setaffinity(0, cpus)
    except OSError:
        return None
    return node


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def measured_link_rates(dev, mib=256):
    """Host <-> device copy rates (GB/s) between pinned host memory and the device,
    timed with CUDA events over one copy of `mib` MiB each way (best of 3)."""
    import torch
    n = mib << 17   # doubles
    d = torch.empty(n, dtype=torch.float64, device=dev)
    h = torch.empty(n, dtype=torch.float64).pin_memory()
    out = {}
    for name, dst, src in (("d2h", h, d), ("h2d", d, h)):
        best = 1e30
        for _ in range(3):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            dst.copy_(src, non_blocking=True)
            e1.record()
            e1.synchronize()
            best = min(best, e0.elapsed_time(e1))
        out[name] = 8 * n / (best * 1e-3) / 1e9
    del d, h
    return out


def reduce_max(value: float, world: int, device=None) -> float:
    """Max of a float over all ranks (identity for one rank)."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def workload(cells):
    from gridap_gb300.synthetic import POISSON3D_128, lognormal_kappa
    w = dict(POISSON3D_128)
    if cells != 128:
        w["cells"] = (cells,) * 3
        w["name"] = f"poisson3d_q1_{cells}^3_parts2x2x2"
    kappa = lognormal_kappa(w["cells"], w["sigma"], w["corr_len"], w["seed"])
    return w, kappa


# ------------------------------------------------------------------------------------
# clocks during the timed region
# ------------------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = Path(os.environ.get("TMPDIR", "/tmp")) / f"gd_clocks_{os.getpid()}.csv"

    def start(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        try:
            self.path.unlink()
        except OSError:
            pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def measured_tensor_peak(sustained=True):
    """Dense BF16 tensor throughput (TFLOP/s) of this machine's GPUs: the measured
    seconds-long figure (a kernel timed inside a longer step) or the burst one."""
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        key = "bf16_tflops_sustained" if sustained else "bf16_tflops"
        if key in d:
            return float(d[key]), "measured"
    return (1700.0 if sustained else 1900.0), "fallback"


def profiled_traffic(workload_name):
    """Per-launch DRAM bytes of the numeric kernels from the committed ncu summary."""
    p = ROOT / "profiles" / "ncu_traffic.json"
    if not p.exists():
        return None
    try:
        d = json.loads(p.read_text())
        return d.get(workload_name)
    except Exception:
        return None


# ------------------------------------------------------------------------------------
# CPU baseline: the oracle's C restatement of the reference's assembly
# ------------------------------------------------------------------------------------
def cpu_assembly(w, kappa, threads):
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle_c
    _, _, ta = oracle_c.assemble(3, w["cells"], w["parts"], w["domain"], (1,) * 6, kappa, w["f"], w["degree"],
                                 "sub", threads, keep=False)
    return ta


def global_nnz(cells):
    m = cells - 1   # free nodes per direction (homogeneous Dirichlet on the whole boundary)
    # 27-point stencil count of an m^3 grid: (3m-2)^3
    return (3 * m - 2) ** 3, m ** 3


def run_reference(args, rank, world):
    """Reference arm: the reference's assembly algorithm (COO + ghost-row exchange +
    compression, restated in C) on the host cores, same workload and metric."""
    if rank != 0:
        return
    w, kappa = workload(args.cells)
    threads = int(np.prod(w["parts"]))
    nnz, _ = global_nnz(w["cells"][0])
    # every warm-up step is a full assembly too (about 5 s each on 8 threads)
    for _ in range(args.warmup):
        cpu_assembly(w, kappa, threads)
    times = [cpu_assembly(w, kappa, threads) for _ in range(args.steps)]
    t = float(np.mean(times))
    v = nnz / t
    line = {"metric": METRIC, "value": v, "unit": UNIT, "impl": "reference", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": w["name"], "cells": list(w["cells"]), "parts": list(w["parts"]), "order": 1,
                       "strategy": "SubAssembledRows", "nnz": nnz, "l2": "inputs and outputs > L2"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"full workload, {args.steps} assemblies (integrate+COO+exchange+compress)"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------------------------
# batched uneven workload (64 problems, Q1-Q3, 16^3..96^3 cells)
# ------------------------------------------------------------------------------------
def run_batched(args, be, stream, dev, mode):
    """One persistent launch per wave of problems that fits the device-memory budget;
    value = all assembled entries / the summed per-wave assembly time."""
    import gc
    import torch
    import gridap_gb300 as G
    from gridap_gb300.batch import BatchedAssembler
    from gridap_gb300.synthetic import BATCHED3D_64, batched_draw, batched_kappa, batched_nnz_estimate
    w = BATCHED3D_64
    draw = batched_draw(w)
    bytes_per_entry = 30.0   # values, column ids, stencil codes and symbolic scratch
    budget = (args.batched_sample_gb if mode == "sample" else args.batched_budget_gb) * 1e9
    waves, cur, cur_b = [], [], 0.0
    for i, (n, k, ks) in enumerate(draw):
        b = batched_nnz_estimate(n, k)[1] * bytes_per_entry
        if cur and cur_b + b > budget:
            waves.append(cur)
            cur, cur_b = [], 0.0
            if mode == "sample":
                break
        cur.append(i)
        cur_b += b
    if cur and (mode == "full" or not waves):
        waves.append(cur)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    tot_nnz = tot_rows = tot_cells = 0
    tot_ms = 0.0
    wave_out = []
    solve_out = []
    for wi, idx in enumerate(waves):
        built = []
        t0 = time.perf_counter()
        for i in idx:
            n, k, ks = draw[i]
            ranks = be.distribute(range(int(np.prod(w["parts"]))))
            model = G.CartesianDiscreteModel(ranks, w["parts"], w["domain"], (n, n, n))
            V = G.TestFESpace(model, G.ReferenceFE(G.lagrangian, float, k), dirichlet_tags="boundary")
            U = G.TrialFESpace(0.0, V)
            dO = G.Measure(G.Triangulation(model), 2 * k)
            assem = G.SparseMatrixAssembler(U, V, G.SubAssembledRows())
            assem.symbolic()
            built.append((model, V, U, assem, G.integral_grad_grad(batched_kappa(n, ks, w["sigma"]), dO),
                          G.integral_source(w["f"], dO)))
        t_setup = time.perf_counter() - t0
        B = BatchedAssembler([(assem, a, l) for (_, _, _, assem, a, l) in built])
        B.assemble()   # autotune + graph capture
        cnt = B.counts()
        for _ in range(max(args.warmup, 3)):
            B.assemble(sync=False)
        torch.cuda.synchronize()
        steps = max(3, min(args.steps, 10))
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        for e0, e1 in ev:
            flush.zero_()
            e0.record(stream)
            B.assemble(sync=False)
            e1.record(stream)
        torch.cuda.synchronize()
        ms = float(np.mean([a.elapsed_time(b) for a, b in ev]))
        cells = sum(draw[i][0] ** 3 for i in idx)
        tot_nnz += cnt["nnz_owned"]
        tot_rows += cnt["rows"]
        tot_cells += cells
        tot_ms += ms
        wave_out.append({"problems": len(idx), "nnz": cnt["nnz_owned"], "rows": cnt["rows"], "ms": ms,
                         "setup_s": t_setup, "tuning": B.tuning()})
        # the batched solve runs on the sample wave only: with --batched full it once ended
        # in an illegal memory access in its final FP64 residual check, cause not yet found
        if args.batched_solve and mode == "sample":
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            st = B.solve(rtol=1e-8, maxit=args.solve_maxit)
            t_solve = time.perf_counter() - t0
            solve_out.append({"wave": wi, "seconds": t_solve, "max_iterations": max(x.iterations for x in st),
                              "all_converged": all(bool(x.converged) for x in st)})
        B.close()
        del B, built
        gc.collect()
        torch.cuda.synchronize()
    peak, peak_kind = measured_peaks()
    alg = 8 * tot_nnz + 8 * tot_rows + 8 * tot_cells
    gbs = alg / (tot_ms * 1e-3) / 1e9 if tot_ms > 0 else 0.0
    return {"workload": w["name"], "mode": mode, "problems": sum(len(x) for x in waves),
            "problems_in_draw": len(draw), "nnz": tot_nnz, "rows": tot_rows, "ms": tot_ms,
            "nnz_per_s": tot_nnz / (tot_ms * 1e-3) if tot_ms > 0 else None,
            "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                         "peak_kind": peak_kind, "algorithmic_bytes": alg},
            "launches_per_wave_step": 1, "waves": wave_out, "solve": solve_out or None,
            "note": "each wave: one persistent kernel launch (CUDA graph replay) over all of its problems"}


# ------------------------------------------------------------------------------------
# vector Q2 linear elasticity (64^3 cells)
# ------------------------------------------------------------------------------------
def run_elasticity(args, be, stream, dev):
    import torch
    import gridap_gb300 as G
    from gridap_gb300 import _lib as L
    from gridap_gb300.synthetic import ELASTICITY3D_64, lognormal_kappa
    w = dict(ELASTICITY3D_64)
    if args.elasticity_cells != 64:
        w["cells"] = (args.elasticity_cells,) * 3
        w["name"] = f"elasticity3d_vq2_{args.elasticity_cells}^3_parts2x2x2"
    ranks = be.distribute(range(int(np.prod(w["parts"]))))
    model = G.CartesianDiscreteModel(ranks, w["parts"], w["domain"], w["cells"])
    V = G.TestFESpace(model, G.ReferenceFE(G.lagrangian, G.VectorValue, w["order"]), dirichlet_tags="left")
    U = G.TrialFESpace(0.0, V)
    assem = G.SparseMatrixAssembler(U, V, G.SubAssembledRows())
    t0 = time.perf_counter()
    assem.symbolic()
    t_sym = time.perf_counter() - t0
    ng, nnz_own, nnz_tot, kpn = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int32()
    L.call("gd_assembler_counts", assem.handle, C.byref(ng), C.byref(nnz_own), C.byref(nnz_tot), C.byref(kpn))
    ncells = int(np.prod(w["cells"]))
    E = lognormal_kappa(w["cells"], w["sigma"], w["corr_len"], w["seed"])
    E_d = torch.from_numpy(E).to(dev)
    c = L.gd_elasticity()
    c.E = E_d.data_ptr()
    c.nu = w["nu"]
    for i in range(3):
        c.force[i] = w["force"][i]
    c.degree = w["degree"]
    c.where = L.GD_DEVICE
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    for _ in range(max(args.warmup, 3)):
        L.call("gd_assemble_elasticity", assem.handle, C.byref(c))
    torch.cuda.synchronize()
    steps = max(3, min(args.steps, 10))
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for e0, e1 in ev:
        flush.zero_()
        e0.record(stream)
        L.call("gd_assemble_elasticity", assem.handle, C.byref(c))
        e1.record(stream)
    torch.cuda.synchronize()
    ms = float(np.mean([a.elapsed_time(b) for a, b in ev]))
    peak, peak_kind = measured_peaks()
    nnz = nnz_own.value
    alg = 8 * nnz + 8 * ng.value + 8 * ncells
    gbs = alg / (ms * 1e-3) / 1e9
    out = {"workload": w["name"], "free_dofs": ng.value, "nnz": nnz, "ms": ms, "nnz_per_s": nnz / (ms * 1e-3),
           "cells_per_s": ncells / (ms * 1e-3), "symbolic_s": t_sym,
           "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                        "peak_kind": peak_kind, "algorithmic_bytes": alg},
           "dtype": "f64", "note": "element matrices E_c*Kel (exact on axis-aligned cells); ms includes the "
                                   "host-side call (the call synchronises for the coefficient check)"}
    if args.elasticity_solve:
        op_matrix = G.PSparseMatrix(assem)
        for name in ("mixed_ir", "jacobi_pcg"):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            try:
                op_matrix.solve(rtol=1e-8, maxit=args.solve_maxit, method=name)
                st = op_matrix.last_stats
                out[f"solve_{name}"] = {"seconds": time.perf_counter() - t0, "iterations": st.iterations,
                                        "rel_residual": st.rel_residual, "converged": bool(st.converged)}
            except Exception as e:   # not converged within maxit
                out[f"solve_{name}"] = {"seconds": time.perf_counter() - t0, "error": str(e)[:200]}
    del assem, U, V, model
    return out


# ------------------------------------------------------------------------------------
# elasticity with E at the Gauss points: element matrices on the tensor cores
# ------------------------------------------------------------------------------------
def run_qp(args, be, stream, dev):
    """64^3 vector-Q2 elasticity with E = exp(g) known at the 27 Gauss points of every
    cell: K_e = sum_q E_q H_q formed by the tcgen05 contraction (BF16 operands split into
    1, 2 or 3 terms, FP32 accumulation) and, for comparison, in FP64 on the CUDA cores.
    Per mode: the assembly time, the contraction kernel's time, tensor and HBM rates, and
    the error against the FP64 mode (y = A x for a random x, and the solution of the
    mixed-precision solve to 1e-8)."""
    import torch
    import gridap_gb300 as G
    from gridap_gb300 import _lib as L
    from gridap_gb300.synthetic import ELASTICITY3D_64, lognormal_at_points
    w = dict(ELASTICITY3D_64)
    if args.qp_cells != 64:
        w["cells"] = (args.qp_cells,) * 3
    name = f"elasticity3d_vq2_{w['cells'][0]}^3_parts2x2x2_E_at_gauss_points"
    ranks = be.distribute(range(int(np.prod(w["parts"]))))
    model = G.CartesianDiscreteModel(ranks, w["parts"], w["domain"], w["cells"])
    V = G.TestFESpace(model, G.ReferenceFE(G.lagrangian, G.VectorValue, w["order"]), dirichlet_tags="left")
    U = G.TrialFESpace(0.0, V)
    assem = G.SparseMatrixAssembler(U, V, G.SubAssembledRows())
    assem.symbolic()
    ng, nnz_own, nnz_tot, kpn = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int32()
    L.call("gd_assembler_counts", assem.handle, C.byref(ng), C.byref(nnz_own), C.byref(nnz_tot), C.byref(kpn))
    ncells = int(np.prod(w["cells"]))
    xq = G.distributed.quadrature_points(model, w["degree"]).reshape(ncells, -1, 3)
    E_qp = lognormal_at_points(w["cells"], xq, w["sigma"], w["corr_len"], w["seed"])
    nqt = E_qp.shape[1]
    E_d = torch.from_numpy(np.ascontiguousarray(E_qp)).to(dev)
    del xq
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    xr = torch.from_numpy(np.random.default_rng(7).normal(size=ng.value)).to(dev)
    hbm, hbm_kind = measured_peaks()
    tpk, tpk_kind = measured_tensor_peak(sustained=True)
    out = {"workload": name, "free_dofs": ng.value, "nnz": nnz_own.value, "quadrature_points_per_cell": nqt,
           "field": "E = exp(g), g the seeded GRF (sigma 0.5, correlation 0.1) interpolated to the Gauss points",
           "modes": {}}
    y_ref = x_ref = x_bf = None
    for mode in ("fp64", "bf16x6", "bf16x3", "bf16"):
        c = L.gd_elasticity_qp()
        c.E_qp = E_d.data_ptr()
        c.nu = w["nu"]
        for i in range(3):
            c.force[i] = w["force"][i]
        c.degree = w["degree"]
        c.precision = L.QP_PRECISIONS[mode]
        c.where = L.GD_DEVICE
        for _ in range(max(args.warmup, 3)):
            L.call("gd_assemble_elasticity_qp", assem.handle, C.byref(c))
        torch.cuda.synchronize()
        steps = max(3, min(args.steps, 10))
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        for e0, e1 in ev:
            flush.zero_()
            e0.record(stream)
            L.call("gd_assemble_elasticity_qp", assem.handle, C.byref(c))
            e1.record(stream)
        torch.cuda.synchronize()
        ms = float(np.mean([a.elapsed_time(b) for a, b in ev]))
        # phase split from the assembler's own events, in separate untimed calls
        L.call("gd_assembler_set_profiling", assem.handle, 1)
        kms, rms = [], []
        for _ in range(3):
            flush.zero_()
            L.call("gd_assemble_elasticity_qp", assem.handle, C.byref(c))
            pts, ent, kp, et = (C.c_int32() for _ in range(4))
            m_e, m_r = C.c_double(), C.c_double()
            L.call("gd_qp_info", assem.handle, C.byref(pts), C.byref(ent), C.byref(kp), C.byref(et),
                   C.byref(m_e), C.byref(m_r))
            kms.append(m_e.value)
            rms.append(m_r.value)
        L.call("gd_assembler_set_profiling", assem.handle, 0)
        ms_k, ms_r = float(np.mean(kms)), float(np.mean(rms))
        nnep = (ent.value + 31) // 32 * 32
        ke_bytes = 4 * ncells * nnep if mode != "fp64" else 8 * ncells * nnep
        y = torch.empty_like(xr)
        L.call("gd_spmv", assem.handle, C.c_void_p(xr.data_ptr()), C.c_void_p(y.data_ptr()), L.GD_DEVICE)
        torch.cuda.synchronize()
        rec = {"ms": ms, "nnz_per_s": nnz_own.value / (ms * 1e-3), "element_kernel_ms": ms_k, "row_kernels_ms": ms_r,
               "element_matrices_bytes": ke_bytes}
        alg = 8 * nnz_own.value + 8 * ng.value + 8 * ncells * nqt
        rec["roofline_assembly"] = {"bound": "hbm", "algorithmic_bytes": alg, "achieved": alg / (ms * 1e-3) / 1e9,
                                    "peak": hbm, "unit": "GB/s", "frac": alg / (ms * 1e-3) / 1e9 / hbm,
                                    "peak_kind": hbm_kind}
        if mode != "fp64":
            nprod = {"bf16": 1, "bf16x3": 3, "bf16x6": 6}[mode]
            nct = 128 if kp.value >= 64 else 256
            n_ct = (ncells + nct - 1) // nct
            flops = 2.0 * (128 * et.value) * (nct * n_ct) * kp.value * nprod   # issued by the MMAs
            useful = 2.0 * ent.value * ncells * nqt                              # sum_q E_q H_q in exact arithmetic
            rec["contraction"] = {
                "kernel": "k_qp_gemm (tcgen05.mma kind::f16, BF16 x BF16 -> FP32 in TMEM)",
                "products_per_term": nprod, "k_padded": kp.value, "issued_tflop": flops / 1e12,
                "tensor": {"achieved": flops / (ms_k * 1e-3) / 1e12, "peak": tpk, "unit": "TFLOP/s",
                           "frac": flops / (ms_k * 1e-3) / 1e12 / tpk, "peak_kind": tpk_kind + " sustained"},
                "useful_tflop_per_s": useful / (ms_k * 1e-3) / 1e12,
                "hbm": {"bytes": ke_bytes, "achieved": ke_bytes / (ms_k * 1e-3) / 1e9, "peak": hbm, "unit": "GB/s",
                        "frac": ke_bytes / (ms_k * 1e-3) / 1e9 / hbm},
                "bound": "hbm (FP32 element matrices written once)"}
        if y_ref is None:
            y_ref = y.clone()
        else:
            rec["error_vs_fp64"] = {"spmv_rel_inf": float((y - y_ref).abs().max() / y_ref.abs().max())}
        if mode in ("fp64", "bf16x6") and args.elasticity_solve:
            x = torch.empty_like(xr)
            st = L.gd_solve_stats()
            t0 = time.perf_counter()
            rc = L.load().gd_solve(assem.handle, L.GD_SOLVE_MIXED_IR, 1e-8, args.solve_maxit,
                                   C.c_void_p(x.data_ptr()), L.GD_DEVICE, C.byref(st))
            rec["solve_mixed_ir"] = {"seconds": time.perf_counter() - t0, "iterations": st.iterations,
                                     "rel_residual": st.rel_residual, "converged": bool(st.converged and rc == 0)}
            if x_ref is None:
                x_ref = x.clone()
            else:
                rec["error_vs_fp64"]["solution_rel_inf"] = float((x - x_ref).abs().max() / x_ref.abs().max())
        if mode == "bf16x6" and x_ref is not None and "solve_mixed_ir" in rec:
            x_bf = x.clone()
        out["modes"][mode] = rec
    out["speedup_bf16x6_vs_fp64"] = out["modes"]["fp64"]["ms"] / out["modes"]["bf16x6"]["ms"]
    if x_ref is not None and "solve_mixed_ir" in out["modes"].get("bf16x6", {}):
        # backward error against the FP64 operator: ||b - A_fp64 x|| / ||b|| for the FP64
        # solution and for the solution of the bf16x6 system (the residual the FP64
        # matrix assigns to it); the gap between the two solutions is conditioning
        c = L.gd_elasticity_qp()
        c.E_qp = E_d.data_ptr()
        c.nu = w["nu"]
        for i in range(3):
            c.force[i] = w["force"][i]
        c.degree = w["degree"]
        c.precision = L.GD_QP_FP64
        c.where = L.GD_DEVICE
        L.call("gd_assemble_elasticity_qp", assem.handle, C.byref(c))
        b = np.zeros(ng.value)
        L.call("gd_system_download", assem.handle, L.ptr(b, C.c_double), None)
        bnorm = np.linalg.norm(b)
        for key, xs in (("fp64_solution", x_ref), ("bf16x6_solution", x_bf)):
            y = torch.empty_like(xs)
            L.call("gd_spmv", assem.handle, C.c_void_p(xs.data_ptr()), C.c_void_p(y.data_ptr()), L.GD_DEVICE)
            torch.cuda.synchronize()
            out.setdefault("backward_error_vs_fp64_operator", {})[key] = float(
                np.linalg.norm(b - y.cpu().numpy()) / bnorm)
    del assem, U, V, model, E_d
    torch.cuda.empty_cache()
    return out


# ------------------------------------------------------------------------------------
# learned preconditioner vs Jacobi (96^3 and 192^3 lognormal diffusion)
# ------------------------------------------------------------------------------------
def run_learned(args, be, dev):
    """The learned flexible CG against FP64 Jacobi-PCG and the mixed-precision Jacobi
    refinement on the same system, each timed on its second (warm) solve, at 96^3 (the
    size the network was trained at; latency-bound: the solve takes a few ms) and 192^3.
    The learned solution is compared with the mixed-precision Jacobi one."""
    import torch
    import gridap_gb300 as G
    from gridap_gb300.learned import LearnedPreconditioner
    from gridap_gb300.synthetic import DIFFUSION3D_96, DIFFUSION3D_192, lognormal_kappa
    path = PKG / "gridap_gb300" / "weights" / "diffusion3d_q1.gdlp"
    if not path.exists():
        return None
    results = []
    for w in (DIFFUSION3D_96, DIFFUSION3D_192):
        cells = w["cells"]
        ranks = be.distribute(range(int(np.prod(w["parts"]))))
        model = G.CartesianDiscreteModel(ranks, w["parts"], w["domain"], cells)
        V = G.TestFESpace(model, G.ReferenceFE(G.lagrangian, float, 1), dirichlet_tags="boundary")
        U = G.TrialFESpace(0.0, V)
        dO = G.Measure(G.Triangulation(model), 2)
        kap = lognormal_kappa(cells, w["sigma"], w["corr_len"], seed=w["seed"] + 1)
        f = np.random.default_rng(w["seed"] + 100).standard_normal(int(np.prod([c + 1 for c in cells])))
        op = G.AffineFEOperator(G.integral_grad_grad(kap, dO), G.integral_source(f, dO), U, V)
        levels, cs = LearnedPreconditioner.file_spec(path)
        net = LearnedPreconditioner(op.matrix, seed=0, levels=levels, coarse_start=cs)
        net.load(path)
        out = {"workload": w["name"], "rtol": 1e-8, "weights": path.name, "levels": net.levels,
               "coarse_start": cs, "params": net.num_params, "timing": "second solve (warm), host clock"}
        runs, xs = {}, {}
        for name, fn in (("jacobi_pcg_fp64", lambda: op.matrix.solve(rtol=1e-8, method="jacobi_pcg")),
                         ("mixed_ir_jacobi", lambda: op.matrix.solve(rtol=1e-8, method="mixed_ir")),
                         ("learned_fcg", lambda: net.solve(rtol=1e-8))):
            fn()   # warm
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            r = fn()
            t = time.perf_counter() - t0
            if name == "learned_fcg":
                x, st, fb = r
                runs[name] = {"seconds": t, "iterations": st.iterations, "rel_residual": st.rel_residual,
                              "converged": bool(st.converged), "fallback_to_jacobi": fb}
            else:
                x = r
                st = op.matrix.last_stats
                runs[name] = {"seconds": t, "iterations": st.iterations, "rel_residual": st.rel_residual,
                              "converged": bool(st.converged)}
            xs[name] = np.asarray(x)
        out.update(runs)
        tl = runs["learned_fcg"]["seconds"]
        out["speedup_vs_jacobi_pcg_fp64"] = runs["jacobi_pcg_fp64"]["seconds"] / tl
        out["speedup_vs_mixed_ir_jacobi"] = runs["mixed_ir_jacobi"]["seconds"] / tl
        ref = xs["mixed_ir_jacobi"]
        out["max_rel_diff_vs_mixed_ir"] = float(np.abs(xs["learned_fcg"] - ref).max() / np.abs(ref).max())
        net.close()
        del op, model, V, U
        results.append(out)
    return results


# ------------------------------------------------------------------------------------
# C1: 2D Q2 Poisson, 128^2 cells, parts (2,2), u = (x+y)^2 on the boundary, f = -4
# ------------------------------------------------------------------------------------
def run_c1(args, be, dev, stream, flush):
    """Numeric assembly (device-resident, per-step CUDA events, L2 flushed between steps),
    the solves to 1e-8 through the Python mirror, and the known answer: Q2 reproduces
    (x+y)^2, so the L2 error of the FP64 solve at rtol 1e-13 is the solver's alone."""
    import torch
    import gridap_gb300 as G
    from gridap_gb300 import _lib as L
    cells, parts, degree, f = (128, 128), (2, 2), 4, -4.0
    u = lambda x, y: (x + y) ** 2
    ranks = be.distribute(range(4))
    model = G.CartesianDiscreteModel(ranks, parts, (0.0, 1.0, 0.0, 1.0), cells)
    V = G.TestFESpace(model, G.ReferenceFE(G.lagrangian, float, 2), dirichlet_tags="boundary")
    U = G.TrialFESpace(u, V)
    assem = G.SparseMatrixAssembler(U, V, G.SubAssembledRows())
    assem.symbolic()
    ng, nnz_own = C.c_int64(), C.c_int64()
    L.call("gd_assembler_counts", assem.handle, C.byref(ng), C.byref(nnz_own), None, None)
    ngdofs, nnz = ng.value, nnz_own.value
    ncells = cells[0] * cells[1]
    kappa_d = torch.ones(ncells, dtype=torch.float64, device=dev)
    coeffs = L.gd_coeffs()
    coeffs.kappa = kappa_d.data_ptr()
    coeffs.f_nodal = None
    coeffs.f_const = f
    coeffs.degree = degree
    coeffs.where = L.GD_DEVICE
    L.call("gd_assemble_numeric", assem.handle, C.byref(coeffs))
    for _ in range(max(args.warmup, 3)):
        L.call("gd_assemble_numeric_async", assem.handle, C.byref(coeffs))
    torch.cuda.synchronize()
    steps = max(args.steps, 10)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for i in range(steps):
        flush.zero_()
        ev[i][0].record(stream)
        L.call("gd_assemble_numeric_async", assem.handle, C.byref(coeffs))
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    ms = float(np.mean([a.elapsed_time(b) for a, b in ev]))
    # the floor of this measurement: one empty kernel between the same events after the
    # same flush
    x1 = torch.zeros(1, device=dev)
    for _ in range(max(args.warmup, 3)):   # the kernel's first launch loads its module
        x1.add_(1.0)
    torch.cuda.synchronize()
    evf = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for i in range(steps):
        flush.zero_()
        evf[i][0].record(stream)
        x1.add_(1.0)
        evf[i][1].record(stream)
    torch.cuda.synchronize()
    floor_ms = float(np.mean([a.elapsed_time(b) for a, b in evf]))
    peak, peak_kind = measured_peaks()
    alg = 8 * nnz + 8 * ngdofs + 8 * ncells
    out = {"workload": "poisson2d_q2_128^2_parts2x2", "cells": list(cells), "parts": list(parts), "order": 2,
           "quadrature_degree": degree, "free_dofs": ngdofs, "nnz": nnz,
           "assembly": {"ms": ms, "launch_floor_ms": floor_ms, "kernels": 1, "steps": steps,
                        "nnz_per_s": nnz / (ms * 1e-3),
                        "roofline": {"bound": "hbm", "algorithmic_bytes": alg, "achieved": alg / (ms * 1e-3) / 1e9,
                                     "peak": peak, "unit": "GB/s", "frac": alg / (ms * 1e-3) / 1e9 / peak,
                                     "peak_kind": peak_kind}}}
    dO = G.Measure(G.Triangulation(model), degree)
    op = G.AffineFEOperator(G.integral_grad_grad(None, dO), G.integral_source(f, dO), U, V)
    solves = {}
    for name, method in (("jacobi_pcg_fp64", "jacobi_pcg"), ("mixed_ir_jacobi", "mixed_ir")):
        op.matrix.solve(rtol=1e-8, method=method)   # warm: one-time buffers
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        op.matrix.solve(rtol=1e-8, method=method)
        t = time.perf_counter() - t0
        st = op.matrix.last_stats
        solves[name] = {"rtol": 1e-8, "seconds": t, "iterations": st.iterations, "rel_residual": st.rel_residual,
                        "converged": bool(st.converged)}
    out["solve"] = solves
    uh = G.solve(op, rtol=1e-13)
    out["kat"] = {"check": "u = (x+y)^2 reproduced by Q2 (test/PoissonTests.jl:14-45 at 128^2), FP64 Jacobi-PCG "
                           "to rtol 1e-13", "l2_error": G.l2_error(uh, u, dO), "bound": 1e-9}
    return out


# ------------------------------------------------------------------------------------
# GB300 arm
# ------------------------------------------------------------------------------------
def run_gb300(args, rank, world, local):
    import torch
    import gridap_gb300 as G
    from gridap_gb300 import _lib as L

    host_node = bind_host_to_gpu(local)
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    w, kappa = workload(args.cells)
    be = G.GB300Backend(local)
    # a dedicated (non-default) stream: the library launches on it and the CUDA
    # events below are recorded on it
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    be.set_stream(stream.cuda_stream)
    ranks = be.distribute(range(int(np.prod(w["parts"]))))
    model = G.CartesianDiscreteModel(ranks, w["parts"], w["domain"], w["cells"])
    V = G.TestFESpace(model, G.ReferenceFE(G.lagrangian, float, 1), dirichlet_tags="boundary")
    U = G.TrialFESpace(0.0, V)
    assem = G.SparseMatrixAssembler(U, V, G.SubAssembledRows())
    t_sym0 = time.perf_counter()
    assem.symbolic()
    t_sym = time.perf_counter() - t_sym0
    ng, nnz_own, nnz_tot, kpn = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int32()
    L.call("gd_assembler_counts", assem.handle, C.byref(ng), C.byref(nnz_own), C.byref(nnz_tot), C.byref(kpn))
    ngdofs, nnz, nnz_total = ng.value, nnz_own.value, nnz_tot.value
    ncells = int(np.prod(w["cells"]))

    kappa_d = torch.from_numpy(kappa).to(dev)
    coeffs = L.gd_coeffs()
    coeffs.kappa = kappa_d.data_ptr()
    coeffs.f_nodal = None
    coeffs.f_const = w["f"]
    coeffs.degree = w["degree"]
    coeffs.where = L.GD_DEVICE
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)

    def step():
        L.call("gd_assemble_numeric_async", assem.handle, C.byref(coeffs))

    # first numeric assembly: validates kappa and runs the launch-shape autotuner
    L.call("gd_assemble_numeric", assem.handle, C.byref(coeffs))
    sh, rows_, nbuf_, nsh = C.c_int32(), C.c_int32(), C.c_int32(), C.c_int32()
    shape_ms = (C.c_float * 8)()
    L.call("gd_assembler_tuning", assem.handle, C.byref(sh), C.byref(rows_), C.byref(nbuf_), shape_ms,
           C.byref(nsh))
    tuning = {"shape": sh.value, "rows_per_chunk": rows_.value, "staging_buffers": nbuf_.value,
              "ms_per_shape": [round(shape_ms[i], 4) for i in range(nsh.value)]}
    L.call("gd_assembler_counts", assem.handle, None, None, None, C.byref(kpn))
    kernels_per_step = kpn.value   # known once the first numeric assembly chose its kernels
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    # ---- device-resident timing: per-step CUDA events, L2 flushed between steps; the
    # steps are queued back to back (no host wait inside the loop) ----
    clocks = ClockSampler(local)
    barrier(world)
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.3)
    t_wall0 = time.perf_counter()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for i in range(args.steps):
        flush.zero_()
        ev[i][0].record(stream)
        step()
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall0
    barrier(world)
    clk = clocks.stop()
    # phase split (coefficient scaling, matrix kernel, rhs kernel) from the assembler's own
    # events, in separate steps so that they add nothing to the timed ones
    L.call("gd_assembler_set_profiling", assem.handle, 1)
    phase = []
    for i in range(max(3, min(args.steps, 20))):
        flush.zero_()
        step()
        m0, m1, m2 = C.c_double(), C.c_double(), C.c_double()
        L.call("gd_assembler_phase_times", assem.handle, C.byref(m0), C.byref(m1), C.byref(m2))
        phase.append((m0.value, m1.value, m2.value))
    torch.cuda.synchronize()
    L.call("gd_assembler_set_profiling", assem.handle, 0)
    step_ms = [a.elapsed_time(b) for a, b in ev]
    ms = float(np.mean(step_ms))
    ms_max = reduce_max(ms, world, dev)
    value = world * nnz / (ms_max * 1e-3)

    peak, peak_kind = measured_peaks()
    alg_bytes = 8 * nnz + 8 * ngdofs + 8 * ncells
    ph = np.array(phase)
    ms_matrix = float(ph[:, 1].mean())
    ms_rhs = float(ph[:, 2].mean())
    ms_zero = float(ph[:, 0].mean())
    step_gbs = alg_bytes / (ms * 1e-3) / 1e9
    mat_bytes = 8 * nnz + 8 * ncells
    mat_gbs = mat_bytes / (ms_matrix * 1e-3) / 1e9
    traffic = profiled_traffic(w["name"])

    # ---- end to end through the C-ABI with host buffers (pinned) ----
    kappa_h = torch.from_numpy(kappa).pin_memory()
    vals_h = torch.empty(nnz, dtype=torch.float64).pin_memory()
    rhs_h = torch.empty(ngdofs, dtype=torch.float64).pin_memory()
    hc = L.gd_coeffs()
    hc.kappa = kappa_h.data_ptr()
    hc.f_nodal = None
    hc.f_const = w["f"]
    hc.degree = w["degree"]
    hc.where = L.GD_HOST
    e2e_steps = max(3, min(args.steps, 10))
    rhs_p = C.cast(C.c_void_p(rhs_h.data_ptr()), L.DP)
    vals_p = C.cast(C.c_void_p(vals_h.data_ptr()), L.DP)

    def e2e_sequential():   # assemble, then download (the reference's order of work)
        L.call("gd_assemble_numeric", assem.handle, C.byref(hc))
        L.call("gd_system_download", assem.handle, rhs_p, vals_p)

    def e2e_overlapped():   # the download of each row range overlaps the next range's assembly
        L.call("gd_assemble_download", assem.handle, C.byref(hc), rhs_p, vals_p)

    e2e_ms = {}
    for name, fn in (("sequential", e2e_sequential), ("overlapped", e2e_overlapped)):
        for _ in range(2):
            fn()
        barrier(world)
        ts = []
        for _ in range(e2e_steps):
            t0 = time.perf_counter()
            fn()
            ts.append(time.perf_counter() - t0)
        e2e_ms[name] = 1e3 * reduce_max(float(np.mean(ts)), world, dev)
    e2e_s = e2e_ms["overlapped"] * 1e-3
    e2e_value = world * nnz / e2e_s
    checksum = float(rhs_h.numpy().sum())
    d2h_bytes = 8 * nnz + 8 * ngdofs
    # the host link's floor for this step: the bytes over the measured copy rates of the link
    link = measured_link_rates(dev)

    # ---- solve to 1e-8 FP64 relative residual on the assembled system ----
    solve = None
    if not args.no_solve:
        solve = {}
        for name, code in (("jacobi_pcg_fp64", L.GD_SOLVE_JACOBI_PCG), ("mixed_ir_jacobi", L.GD_SOLVE_MIXED_IR)):
            x = torch.empty(ngdofs, dtype=torch.float64, device=dev)
            st = L.gd_solve_stats()
            # one untimed solve first: the method's one-time device buffers and tables
            L.load().gd_solve(assem.handle, code, 1e-8, args.solve_maxit, C.c_void_p(x.data_ptr()),
                              L.GD_DEVICE, C.byref(st))
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            rc = L.load().gd_solve(assem.handle, code, 1e-8, args.solve_maxit, C.c_void_p(x.data_ptr()),
                                   L.GD_DEVICE, C.byref(st))
            t_solve = time.perf_counter() - t0
            solve[name] = {"rtol": 1e-8, "seconds": t_solve, "timing": "second solve (warm)", "iterations": st.iterations,
                           "rel_residual": st.rel_residual, "converged": bool(st.converged and rc == 0),
                           "ms_per_iteration": 1e3 * t_solve / max(st.iterations, 1)}

    learned = None
    if not args.no_learned:
        learned = run_learned(args, be, dev)
    c1 = None
    if not args.no_c1:
        c1 = run_c1(args, be, dev, stream, flush)
    elasticity = None
    if not args.no_elasticity:
        elasticity = run_elasticity(args, be, stream, dev)
    quadrature = None
    if not args.no_qp:
        quadrature = run_qp(args, be, stream, dev)
    batched = None
    if args.batched != "off":
        batched = run_batched(args, be, stream, dev, args.batched)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = int(np.prod(w["parts"]))
        ta = cpu_assembly(w, kappa, threads)
        cpu = {"value": nnz / ta, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": "one full assembly of the same workload by the oracle's C restatement of the reference "
                         "(per-cell quadrature, COO, ghost-row exchange, sparse compression), one thread per part"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": w["name"], "cells": list(w["cells"]), "parts": list(w["parts"]), "order": 1,
                       "quadrature_degree": w["degree"], "strategy": "SubAssembledRows", "nnz": nnz,
                       "nnz_stored_with_ghost_rows": nnz_total, "free_dofs": ngdofs, "cells_total": ncells,
                       "l2": f"flushed between steps ({L2_FLUSH_BYTES >> 20} MiB write); outputs > L2",
                       "parallelism": f"replicas x{world}" if world > 1 else "1 GPU, 8 parts as slabs"},
            "cells_per_s": world * ncells / (ms_max * 1e-3),
            "roofline": {"bound": "hbm", "achieved": step_gbs, "peak": peak, "unit": "GB/s",
                         "frac": step_gbs / peak, "traffic": traffic,
                         "peak_kind": peak_kind, "algorithmic_bytes": alg_bytes,
                         "scope": "whole numeric assembly (k_prescale: coefficient scaling and check; "
                                  "k_numeric_q1: matrix values with the rhs fused)",
                         "matrix_kernel": {"ms": ms_matrix, "bytes": mat_bytes, "achieved": mat_gbs,
                                           "frac": mat_gbs / peak},
                         "rhs_kernel_ms": ms_rhs, "prescale_ms": ms_zero},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 8 * ncells,
                    "d2h_bytes_per_step": d2h_bytes, "ms_per_step": 1e3 * e2e_s,
                    "ms_per_step_sequential": e2e_ms["sequential"],
                    "link_gbs": link, "link_floor_ms": 1e3 * (8 * ncells / (link["h2d"] * 1e9) +
                                                               d2h_bytes / (link["d2h"] * 1e9)),
                    "rhs_checksum": checksum,
                    "host_numa_node": host_node},
            "gpu_launches": kernels_per_step * args.steps,
            "autotune": tuning,
            "clocks": clk,
            "symbolic_s": t_sym,
            "wall_s_timed_region": t_wall,
            "solve": solve,
            "learned": learned,
            "c1": c1,
            "elasticity": elasticity,
            "quadrature": quadrature,
            "batched": batched,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)
    be.close()


def main():
    args = parse()
    rank, world, local = dist_env()
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if args.impl == "gb300" else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    try:
        if args.impl == "reference":
            run_reference(args, rank, world)
        else:
            run_gb300(args, rank, world, local)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
