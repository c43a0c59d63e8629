"""Benchmark: forward solve + adjoint gradient, seconds per 1M DOF.

Workload (the headline configuration): Hexa1 cube of 70 x 70 x 70 elements
(357,911 nodes, 1,073,733 DOF), interior nodes jittered by U(-0.1h, 0.1h)
(seed 0), IsotropicElasticity3D(E=1000, nu=0.3), x=0 face clamped, z-force
-1/n_nodes per node on the x=1 face.  One step = `solve()` to relative
residual 1e-10 plus the gradient of sum(u) with respect to the nodal forces
through the hand-written adjoint (the reference benchmark's loss,
benchmarks/cubes.py:31-37).  Synthetic seeded data; no dataset.

value      mixed precision: FP32 K and FP32 CG with FP64 residual
           replacement, preconditioned by the smoothed-aggregation multigrid
           V-cycle (--precond amg, the library default) or block Jacobi
           (--precond jacobi); inputs resident in HBM, CUDA events on the
           launching stream.
e2e        the same through the public API from host tensors: the model is
           built from CPU tensors, so every step copies its inputs to the
           device and its results (u, f, sigma, F, grad) back.
plain_fp64 the FP64 Jacobi-CG path (scalar CSR in the reference pattern).
mixed_block_jacobi  the mixed path with block Jacobi (the persistent CG
           kernel), reported beside the headline.

`--workload heat` times the heat-conduction path instead (SolidHeat,
steady solve + adjoint gradient w.r.t. the per-element conductivity, FP64
Jacobi CG or mixed multigrid) and `--workload thermal` the reference's own
thermal benchmark (benchmarks/thermal.py: SIMP slab, thermal compliance
gradient w.r.t. the densities); each prints its own line.  The headline is
the elastic cube.

`--impl reference` times the CPU oracle (a restatement of torch-fem's CPU
path: numpy assembly + scipy Jacobi-CG) on a bounded sample of the same
workload, because torch-fem itself is Python that cannot be run where the
GPU is.
"""

from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
for _p in (ROOT, ROOT / "torch-fem_gb300"):
    if str(_p) not in sys.path:
        sys.path.insert(0, str(_p))

import numpy as np  # noqa: E402
import torch  # noqa: E402

METRIC = "solve+grad s per 1M DOF: FP32-CG+FP64-refine+adjoint vs plain FP64 @ rel err 1e-8"
UNIT = "s/1M DOF"


def cube_nodes(n: int):
    """Nodes and elements of the n^3 Hexa1 cube, interior nodes jittered by
    U(-0.1, 0.1)/n per coordinate from torch seed 0."""
    from torchfem_gb300 import mesh

    nodes, el = mesh.cube_hexa(n + 1, n + 1, n + 1)
    gen = torch.Generator().manual_seed(0)
    inner = ((nodes > 0) & (nodes < 1)).all(1)
    nodes = nodes + inner[:, None] * (torch.rand(nodes.shape, generator=gen, dtype=torch.float64) * 2 - 1) * (0.1 / n)
    return nodes, el


def cube_workload(n: int, device):
    """The jittered cube with E = 1000, nu = 0.3, x = 0 clamped and the
    z-force -1/n_nodes on every node of x = 1 (forces returned separately)."""
    from torchfem_gb300 import Solid
    from torchfem_gb300.materials import IsotropicElasticity3D

    nodes, el = cube_nodes(n)
    x0 = nodes[:, 0] == 0.0
    x1 = nodes[:, 0] == 1.0
    nodes, el = nodes.to(device), el.to(device)
    m = Solid(nodes, el, IsotropicElasticity3D(1000.0, 0.3))
    con = torch.zeros(nodes.shape, dtype=torch.bool, device=device)
    con[x0.to(device), :] = True
    m.constraints = con
    forces = torch.zeros(nodes.shape, dtype=torch.float64, device=device)
    forces[x1.to(device), 2] = -1.0 / len(nodes)
    return m, forces


def step(m, forces, precision, stol, precond=None):
    f = forces.detach().requires_grad_(True)
    m.forces = f
    u, fi, s, gr, st = m.solve(stol=stol, precision=precision, differentiable_parameters=f,
                               preconditioner=precond)
    (g,) = torch.autograd.grad(u.sum(), f)
    return u, fi, s, gr, st, g


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.first = threading.Event()
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            # nvidia-smi's own start-up (driver and NVML initialisation) stays
            # outside the timed region: wait for its first sample
            self.first.wait(timeout=10.0)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())
            self.first.set()
        self.first.set()

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for name, val in zip(names, parts[4:8]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak_hbm():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except (KeyError, ValueError):
            pass
    return 6800.0, "fallback"


def cg_iteration_bytes(dm) -> float:
    """Algorithmic bytes of one mixed-precision CG iteration: the FP32 block
    matrix (36 value bytes and one int32 column per stored block, int64 slice
    pointers) and twelve FP32 vector streams (SpMV: p, q; update: x, r read and
    written, p, q read, z written; direction: z, p read, p written) plus the
    3x3 block-Jacobi inverse (12 bytes per DOF)."""
    n_slices = (dm.n_nod + 31) // 32
    return dm.n_blocks * 40 + 8 * (n_slices + 1) + 48 * dm.n_dofs + 12 * dm.n_dofs


def spmv_bytes(dm, value_bytes: int = 4) -> float:
    """Algorithmic bytes of one level-0 block SpMV: d*d values of
    `value_bytes` (4: the FP32 matrix, 2: the FP16 smoothing copy) and one
    int32 column per stored block, x read once, y written once (the padding
    slots of the sliced layout are not counted)."""
    d = dm.d
    return dm.n_blocks * (value_bytes * d * d + 4) + 2 * 4 * dm.n_dofs


def level0_launch_bytes(dm, smoother: str) -> float:
    """Mean algorithmic bytes of the timed level-0 launches of one multigrid
    CG iteration: the four Chebyshev passes (FP16 copy with --smoother fp16)
    and CG's q = A p (always the FP32 matrix)."""
    smooth = spmv_bytes(dm, 2 if smoother == "fp16" else 4)
    return (4 * smooth + spmv_bytes(dm, 4)) / 5


def _port_step(n: int):
    """One solve + adjoint of the oracle port on the jittered n^3 cube:
    (seconds, of which CG seconds, DOF, CG iterations of both solves)."""
    from oracle import fem_oracle as O

    nodes, el = O.cube_hexa(n + 1, n + 1, n + 1)
    rng = torch.Generator().manual_seed(0)
    inner = ((nodes > 0) & (nodes < 1)).all(1)
    jit = (torch.rand(nodes.shape, generator=rng, dtype=torch.float64).numpy() * 2 - 1) * (0.1 / n)
    nodes = nodes + inner[:, None] * jit
    con = np.zeros(nodes.shape, dtype=bool)
    con[nodes[:, 0] == 0.0, :] = True
    F = np.zeros(nodes.shape)
    F[nodes[:, 0] == 1.0, 2] = -1.0 / len(nodes)
    O.LinearModel.cg_iterations.clear()
    O.LinearModel.cg_seconds.clear()
    t0 = time.perf_counter()
    m = O.LinearModel(nodes, el, O.elastic_c("3d", 1000.0, 0.3, len(el)))
    m.solve(F, con, method="cg", rtol=1e-10)
    m.adjoint(np.ones(m.n_dofs), method="cg", rtol=1e-10)
    t = time.perf_counter() - t0
    return t, sum(O.LinearModel.cg_seconds), nodes.size, sum(O.LinearModel.cg_iterations)


def cpu_baseline(n_sample: int, n_target: int = 70):
    """The oracle port (the reference's CPU path restated: numpy assembly,
    scipy Jacobi CG to rtol 1e-10, forward + adjoint) timed on two cubes,
    (2 n_sample / 3)^3 and n_sample^3, then extrapolated to the n_target^3
    workload: set-up (integration, assembly, stresses) by DOF, the CG by
    DOF x iterations, with the iteration growth measured between the two
    samples (Jacobi-CG iterations grow like a power of n, about n^1)."""
    n_small = max(4, (2 * n_sample) // 3)
    t_s, cg_s, dofs_s, it_s = _port_step(n_small)
    t_l, cg_l, dofs_l, it_l = _port_step(n_sample)
    alpha = math.log(it_l / it_s) / math.log(n_sample / n_small) if it_s > 0 and it_l > 0 else 1.0
    dofs_t = 3 * (n_target + 1) ** 3
    it_t = it_l * (n_target / n_sample) ** alpha
    t_t = (t_l - cg_l) * (dofs_t / dofs_l) + cg_l * (dofs_t / dofs_l) * (it_t / it_l)
    return {"value": t_t / (dofs_t / 1e6), "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
            "sample": f"oracle port (numpy assembly + scipy Jacobi-CG, rtol 1e-10, solve + adjoint) on the "
                      f"{n_small}^3 and {n_sample}^3 jittered Hexa1 cubes ({dofs_s} and {dofs_l} DOF: "
                      f"{t_s:.2f} s and {t_l:.2f} s, of which CG {cg_s:.2f} s and {cg_l:.2f} s over {it_s} and "
                      f"{it_l} iterations), extrapolated to {n_target}^3 ({dofs_t} DOF): set-up by DOF, CG by "
                      f"DOF x iterations with iterations ~ n^{alpha:.2f} ({it_t:.0f} predicted); scipy's SpMV "
                      f"runs on one thread, numpy may use every core",
            "samples": {"n": [n_small, n_sample], "seconds": [t_s, t_l], "cg_seconds": [cg_s, cg_l],
                        "cg_iterations": [it_s, it_l], "iteration_exponent": alpha, "predicted_seconds": t_t}}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend)
        return dist, rank, world, local
    return None, rank, world, local


def reduce_max(dist, x: float, device) -> float:
    if dist is None:
        return x
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(args):
    dist, rank, world, _ = dist_setup()
    if rank != 0:
        return
    runs = [cpu_baseline(args.cpu_n, args.n) for _ in range(max(args.warmup, 0) + max(args.steps, 1))]
    timed = runs[args.warmup:] or runs
    v = sum(r["value"] for r in timed) / len(timed)
    cb = dict(timed[-1])
    cb["value"] = v
    # the step time at the full workload is the samples' extrapolation, as the value is
    ms = 1e3 * sum(r["samples"]["predicted_seconds"] for r in timed) / len(timed)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"hexa1_cube_{args.n}^3_jittered (CPU sample {args.cpu_n}^3)",
                   "parallelism": "replicas", "ms_per_step": "extrapolated from the two CPU samples"},
        "cpu_baseline": cb,
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


HEAT_METRIC = "heat solve+grad s per 1M DOF"
THERMAL_METRIC = "thermal SIMP slab fwd+bwd s per 1M DOF (benchmarks/thermal.py)"


def thermal_slab(N: int, device):
    """The slab of the reference's thermal benchmark (benchmarks/thermal.py:
    get_slab): one Hexa1 layer of N x N/2 elements on [0,2]x[0,1], thickness
    2/N, conductivity k = k_max (1e-3 + (1 - 1e-3) rho^3) with rho = 0.5 per
    element, T = 0 on x = 0, unit heat flux per area on x = 2 lumped to the
    nodes with trapezoidal weights."""
    from torchfem_gb300 import SolidHeat, mesh
    from torchfem_gb300.materials import IsotropicConductivity3D

    lx, ly = 2.0, 1.0
    nx, ny, nz = N, N // 2, 1
    lz = lx / nx
    nodes, elements = mesh.cube_hexa(nx + 1, ny + 1, nz + 1, lx, ly, lz)
    right = nodes[:, 0] == lx
    wy = torch.full((len(nodes),), ly / ny, dtype=torch.float64)
    wy[(nodes[:, 1] == 0.0) | (nodes[:, 1] == ly)] /= 2.0
    wz = torch.full((len(nodes),), lz / nz, dtype=torch.float64)
    wz[(nodes[:, 2] == 0.0) | (nodes[:, 2] == lz)] /= 2.0
    q = torch.zeros(len(nodes), 1, dtype=torch.float64)
    q[right, 0] = wy[right] * wz[right]
    left = nodes[:, 0] == 0.0
    model = SolidHeat(nodes.to(device), elements.to(device), IsotropicConductivity3D(1.0))
    model.constraints[left.to(device)] = True
    model.heat_flux = q.to(device)
    rho = torch.full((model.n_elem,), 0.5, dtype=torch.float64, device=device)
    base = model.material.KAPPA.detach().to(device)
    return model, rho, base


def thermal_step(model, base_kappa, rho0, precision, stol):
    """One benchmark repetition: SIMP conductivity of the densities, forward
    solve with them as differentiable parameters, then the backward of the
    thermal compliance q . T."""
    rho = rho0.detach().requires_grad_(True)
    model.material.KAPPA = (1e-3 + (1.0 - 1e-3) * rho**3.0)[:, None, None] * base_kappa
    u, *_ = model.solve(differentiable_parameters=rho, stol=stol, precision=precision)
    compliance = torch.inner(model.heat_flux.ravel(), u.ravel())
    compliance.backward()
    return u, rho.grad


def run_thermal(args):
    """--warmup untimed and --steps timed repetitions of the thermal slab
    benchmark at N = --thermal-n, mixed precision (multigrid) as the value and
    the FP64 Jacobi CG beside it; CUDA events on the launching stream."""
    from torchfem_gb300 import _lib

    dev = torch.device("cuda", 0)
    lib = _lib.load()
    model, rho, base = thermal_slab(args.thermal_n, dev)
    stream = torch.cuda.current_stream(dev)
    for _ in range(max(args.warmup, 0)):
        thermal_step(model, base, rho, "mixed", args.stol)
    torch.cuda.synchronize()
    ms, iters, u_ms, u_n, launches, clocks, (u_m, g_m) = timed_steps(
        lib, lambda: (thermal_step(model, base, rho, "mixed", args.stol), model), args.steps, stream)
    thermal_step(model, base, rho, "fp64", args.stol)
    p_ms, p_iters, p_ums, p_un, _, _, (u_p, g_p) = timed_steps(
        lib, lambda: (thermal_step(model, base, rho, "fp64", args.stol), model), 1, stream)
    dm = model.device_mesh
    n_dofs = model.n_dofs
    roof, roof_plain = scalar_rooflines(lib, dm, n_dofs, (u_ms / u_n) / 1e3 if u_n else None,
                                        (p_ums / p_un) / 1e3 if p_un else None, args.smoother)
    line = {
        "metric": THERMAL_METRIC, "value": ms / 1e3 / (n_dofs / 1e6), "unit": UNIT, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic (the benchmark's slab)",
        "config": {"workload": f"thermal_slab_simp N={args.thermal_n} (benchmarks/thermal.py)",
                   "dofs": n_dofs, "nnz": dm.nnz, "n_elem": model.n_elem, "stol": args.stol,
                   "preconditioner": "smoothed-aggregation multigrid (constant near-null vector)",
                   "fp64_residual": "element pass" if args.residual == "elements" else "FP64 copy of the sliced matrix",
                   "l2": "inputs larger than L2 (FP64 gradient cache %.0f MB)"
                         % ((dm.bt.numel() + dm.detj.numel()) * 8 / 1e6)},
        "cg_iterations": iters, "gpu_launches": launches,
        "roofline": roof,
        "plain_fp64": {"value": p_ms / 1e3 / (n_dofs / 1e6), "ms_per_step": p_ms, "cg_iterations": p_iters,
                       "roofline": roof_plain},
        "mixed_speedup_vs_plain": p_ms / ms,
        "rel_err_mixed_vs_fp64": {"u": float((u_m - u_p).detach().abs().max() / u_p.detach().abs().max()),
                                  "grad": float((g_m - g_p).abs().max() / g_p.abs().max())},
        "clocks": clocks,
    }
    print(json.dumps(line))


def heat_inputs(n: int):
    """The heat cube's inputs: the jittered n^3 Hexa1 mesh (interior nodes
    moved by U(-0.1h, 0.1h), seed 0), conductivity U(1, 2) per element
    (seed 1) and the x = 0 face, as CPU tensors."""
    from torchfem_gb300 import mesh

    nodes, el = mesh.cube_hexa(n + 1, n + 1, n + 1)
    gen = torch.Generator().manual_seed(0)
    inner = ((nodes > 0) & (nodes < 1)).all(1)
    nodes = nodes + inner[:, None] * (torch.rand(nodes.shape, generator=gen, dtype=torch.float64) * 2 - 1) * (0.1 / n)
    kappa = 1.0 + torch.rand(len(el), generator=torch.Generator().manual_seed(1), dtype=torch.float64)
    return nodes, el, kappa, nodes[:, 0] == 0.0


def heat_workload(n: int, device):
    """SolidHeat on the heat cube (heat_inputs), T = 0 on the x = 0 face,
    uniform source 1/n_nodes."""
    from torchfem_gb300 import SolidHeat
    from torchfem_gb300.materials import IsotropicConductivity3D

    nodes, el, kappa, x0 = heat_inputs(n)
    m = SolidHeat(nodes.to(device), el.to(device), IsotropicConductivity3D(kappa.to(device)))
    m.constraints[x0.to(device)] = True
    q = torch.full((len(nodes), 1), 1.0 / len(nodes), dtype=torch.float64, device=device)
    return m, kappa.to(device), q


def heat_step(m, kappa0, q, stol, precision="mixed"):
    from torchfem_gb300.materials import IsotropicConductivity3D

    kappa = kappa0.detach().requires_grad_(True)
    m.material = IsotropicConductivity3D(kappa)
    m.heat_flux = q
    T, f, flux, _, _ = m.solve(stol=stol, precision=precision, differentiable_parameters=kappa)
    (g,) = torch.autograd.grad(T.sum(), kappa)
    return T, g


def _heat_port_step(n: int):
    """One solve + adjoint of the heat oracle on the heat cube of size n:
    (seconds, of which CG seconds, DOF, CG iterations of both solves)."""
    from oracle import heat_oracle as H

    nodes, el, kappa, x0 = (t.numpy() for t in heat_inputs(n))
    H.HeatModel.cg_iterations.clear()
    H.HeatModel.cg_seconds.clear()
    t0 = time.perf_counter()
    om = H.HeatModel(nodes, el, kappa[:, None, None] * np.eye(3))
    om.solve(np.full(len(nodes), 1.0 / len(nodes)), x0, method="cg", rtol=1e-10)
    om.adjoint(np.ones(len(nodes)), method="cg", rtol=1e-10)
    t = time.perf_counter() - t0
    return t, sum(H.HeatModel.cg_seconds), len(nodes), sum(H.HeatModel.cg_iterations)


def heat_cpu_baseline(n_sample: int, n_target: int):
    """The heat oracle's solve + adjoint (numpy assembly, scipy Jacobi-CG to
    1e-10) on two cubes of the same kind, (2 n_sample / 3)^3 and n_sample^3,
    extrapolated to the n_target^3 workload as cpu_baseline does: set-up by
    DOF, the CG by DOF x iterations with the measured iteration growth."""
    n_small = max(4, (2 * n_sample) // 3)
    t_s, cg_s, dofs_s, it_s = _heat_port_step(n_small)
    t_l, cg_l, dofs_l, it_l = _heat_port_step(n_sample)
    alpha = math.log(it_l / it_s) / math.log(n_sample / n_small) if it_s > 0 and it_l > 0 else 1.0
    dofs_t = (n_target + 1) ** 3
    it_t = it_l * (n_target / n_sample) ** alpha
    t_t = (t_l - cg_l) * (dofs_t / dofs_l) + cg_l * (dofs_t / dofs_l) * (it_t / it_l)
    return {"value": t_t / (dofs_t / 1e6), "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
            "sample": f"heat oracle (numpy assembly + scipy Jacobi-CG, rtol 1e-10, solve + adjoint) on the "
                      f"{n_small}^3 and {n_sample}^3 jittered Hexa1 cubes ({dofs_s} and {dofs_l} DOF: {t_s:.2f} s "
                      f"and {t_l:.2f} s, of which CG {cg_s:.2f} s and {cg_l:.2f} s over {it_s} and {it_l} "
                      f"iterations), extrapolated to {n_target}^3 ({dofs_t} DOF): set-up by DOF, CG by DOF x "
                      f"iterations with iterations ~ n^{alpha:.2f} ({it_t:.0f} predicted)",
            "samples": {"n": [n_small, n_sample], "seconds": [t_s, t_l], "cg_seconds": [cg_s, cg_l],
                        "cg_iterations": [it_s, it_l], "iteration_exponent": alpha, "predicted_seconds": t_t}}


def timed_steps(lib, fn, steps, stream):
    """Runs fn() `steps` times between CUDA events on `stream` with the
    library's CG timing on; returns (ms per step, CG iterations per step,
    summed CG unit time in ms, timed units, kernel launches, clock summary,
    the last result)."""
    lib.fem_set_timing(1)
    spmv_ms, spmv_n, iters, out = 0.0, 0, [], None
    launches0 = lib.fem_launch_count()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(stream.device.index or 0) as clocks:
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(steps):
            out, model = fn()
            st = model.last_solve
            iters.append(st.iterations)
            spmv_ms += st.system.stats.spmv_ms
            spmv_n += st.system.stats.spmv_timed
        ev1.record(stream)
        torch.cuda.synchronize()
    launches = lib.fem_launch_count() - launches0
    lib.fem_set_timing(0)
    return ev0.elapsed_time(ev1) / steps, iters, spmv_ms, spmv_n, launches, clocks.summary(), out


def scalar_rooflines(lib, dm, n_dofs, mixed_unit, plain_unit, smoother="fp16"):
    """Roofline objects of the two heat paths: the level-0 SpMVs of the
    multigrid CG (level0_launch_bytes: four smoothing passes on the FP16 copy,
    2-byte value and int32 column per stored entry, and q = A p on the FP32
    matrix, 4-byte value; x read once, y written once) and one FP64
    Jacobi-CG iteration of the persistent
    kernel (8-byte value and int32 column per entry, int64 row pointers,
    twelve FP64 vector streams and the inverse diagonal)."""
    peak, peak_kind = measured_peak_hbm()

    def obj(kernel, sb, unit_s):
        achieved = sb / unit_s / 1e9 if unit_s else None
        return {"bound": "hbm", "kernel": kernel, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": (achieved / peak) if achieved else None, "traffic": None, "algorithmic_bytes": sb,
                "avg_unit_us": unit_s * 1e6 if unit_s else None, "peak_source": peak_kind}

    mixed = obj("k_sell_op1<*> (level-0 scalar SpMVs of the multigrid CG: four smoothing passes on the %s, "
                "q = A p on the FP32 matrix)" % ("FP16 copy" if smoother == "fp16" else "FP32 matrix"),
                level0_launch_bytes(dm, smoother), mixed_unit)
    if lib.fem_get_cg_path() in (1, 2):
        plain = obj("persistent FP64 Jacobi-CG kernel (one iteration)",
                    dm.nnz * 12 + (n_dofs + 1) * 8 + 13 * 8 * n_dofs, plain_unit)
    else:
        plain = obj("k_spmv_csr (FP64 CSR SpMV of the Jacobi CG)",
                    dm.nnz * 12 + (n_dofs + 1) * 8 + 2 * n_dofs * 8, plain_unit)
    return mixed, plain


def run_heat(args):
    """Steady heat conduction on the n^3 cube (n = --heat-n): --warmup
    untimed and --steps timed steps of solve + adjoint in mixed precision
    (multigrid), then the FP64 Jacobi CG on the same problem; CUDA events
    on the launching stream."""
    from torchfem_gb300 import _lib

    dev = torch.device("cuda", 0)
    lib = _lib.load()
    m, kappa, q = heat_workload(args.heat_n, dev)
    stream = torch.cuda.current_stream(dev)
    for _ in range(max(args.warmup, 0)):
        heat_step(m, kappa, q, args.stol, "mixed")
    torch.cuda.synchronize()
    ms, iters, u_ms, u_n, launches, clocks, (T_m, g_m) = timed_steps(
        lib, lambda: (heat_step(m, kappa, q, args.stol, "mixed"), m), args.steps, stream)
    heat_step(m, kappa, q, args.stol, "fp64")
    p_ms, p_iters, p_ums, p_un, _, _, (T_p, g_p) = timed_steps(
        lib, lambda: (heat_step(m, kappa, q, args.stol, "fp64"), m), 1, stream)
    dm = m.device_mesh
    n_dofs = m.n_dofs
    roof, roof_plain = scalar_rooflines(lib, dm, n_dofs, (u_ms / u_n) / 1e3 if u_n else None,
                                        (p_ums / p_un) / 1e3 if p_un else None, args.smoother)
    line = {
        "metric": HEAT_METRIC + " (FP32 multigrid CG + FP64 refinement + adjoint)",
        "value": ms / 1e3 / (n_dofs / 1e6), "unit": UNIT, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic (seeded jittered cube)",
        "config": {"workload": f"solidheat_hexa1_cube_{args.heat_n}^3_jittered_steady_solve+adjoint",
                   "dofs": n_dofs, "nnz": dm.nnz, "n_elem": m.n_elem, "stol": args.stol,
                   "preconditioner": "smoothed-aggregation multigrid (constant near-null vector)",
                   "fp64_residual": "element pass" if args.residual == "elements" else "FP64 copy of the sliced matrix",
                   "l2": "inputs larger than L2 (FP64 K = %.0f MB)" % (dm.nnz * 12 / 1e6)},
        "cg_iterations": iters, "gpu_launches": launches,
        "roofline": roof,
        "plain_fp64": {"value": p_ms / 1e3 / (n_dofs / 1e6), "ms_per_step": p_ms, "cg_iterations": p_iters,
                       "roofline": roof_plain},
        "mixed_speedup_vs_plain": p_ms / ms,
        "rel_err_mixed_vs_fp64": {"T": float((T_m - T_p).detach().abs().max() / T_p.detach().abs().max()),
                                  "grad": float((g_m - g_p).abs().max() / g_p.abs().max())},
        "clocks": clocks,
        "cpu_baseline": heat_cpu_baseline(args.heat_cpu_n, args.heat_n),
    }
    print(json.dumps(line))


ASSEMBLY_METRIC = "assembly solve+grad s per 1M DOF (coupled parts, FP64 Jacobi CG on T^T K T)"


def assembly_workload(n: int, device):
    """Two jittered n^3 Hexa1 cubes tied face to face at x = 1 (interfaces
    unjittered, so the tied nodes coincide), the first clamped at x = 0, and
    a reference point at x = 2.5 driving the far face x = 2 with a moment
    about x and a pull along z.  Returns the assembly, its first part, the
    per-element Young's moduli of that part and the point."""
    from torchfem_gb300 import Assembly, ReferencePoint, Solid
    from torchfem_gb300.materials import IsotropicElasticity3D

    nodes, el = cube_nodes(n)
    nodes_b = nodes.clone()
    nodes_b[:, 0] += 1.0
    E0 = 1000.0 * (1.0 + 0.1 * torch.randn(len(el), generator=torch.Generator().manual_seed(2), dtype=torch.float64))
    a = Solid(nodes.to(device), el.to(device), IsotropicElasticity3D(E0.to(device), 0.3))
    b = Solid(nodes_b.to(device), el.to(device), IsotropicElasticity3D(1000.0, 0.3))
    a.constraints[(nodes[:, 0] == 0.0).to(device)] = True
    point = ReferencePoint([2.5, 0.5, 0.5])
    point.forces[0, 3] = 1.0
    point.forces[0, 2] = 1.0
    asm = Assembly([a, b, point])
    asm.coupling(b, nodes_b[:, 0] == 1.0, a, nodes[:, 0] == 1.0)
    asm.coupling(b, nodes_b[:, 0] == 2.0, point)
    return asm, a, E0.to(device), point


def assembly_step(asm, a, E0, point, stol):
    from torchfem_gb300.materials import IsotropicElasticity3D

    E = E0.detach().requires_grad_(True)
    a.material = IsotropicElasticity3D(E, 0.3)
    u, f, _, _, _ = asm.solve(stol=stol, differentiable_parameters=E)
    w = torch.inner(point.forces.ravel().to(u[2].dtype), u[2].ravel())
    (g,) = torch.autograd.grad(w, E)
    return u, g


def _assembly_port_step(n: int):
    """The assembly oracle's coupled solve (numpy assembly, scipy Jacobi CG to
    1e-10) of the workload at size n: (seconds, CG seconds, DOF, CG iterations)."""
    from oracle import assembly_oracle as A
    from oracle import fem_oracle as O

    nodes, el = (t.numpy() for t in cube_nodes(n))
    nodes_b = nodes.copy()
    nodes_b[:, 0] += 1.0
    E0 = 1000.0 * (1.0 + 0.1 * torch.randn(len(el), generator=torch.Generator().manual_seed(2),
                                           dtype=torch.float64).numpy())
    t0 = time.perf_counter()
    a = A.ModelPart(O.LinearModel(nodes, el, O.elastic_c("3d", E0, 0.3, len(el))), 3)
    b = A.ModelPart(O.LinearModel(nodes_b, el, O.elastic_c("3d", 1000.0, 0.3, len(el))), 3)
    a.constraints[nodes[:, 0] == 0.0] = True
    point = A.PointPart([2.5, 0.5, 0.5])
    point.forces[0, 3] = 1.0
    point.forces[0, 2] = 1.0
    asm = A.AssemblyOracle([a, b, point])
    asm.coupling(1, nodes_b[:, 0] == 1.0, 0, nodes[:, 0] == 1.0)
    asm.coupling(1, nodes_b[:, 0] == 2.0, 2)
    tc = time.perf_counter()
    asm.solve(method="cg", rtol=1e-10)
    t_cg = time.perf_counter() - tc
    its = asm.cg_iterations
    # the adjoint: one more solve of the same symmetric system
    t = time.perf_counter() - t0 + t_cg
    return t, 2 * t_cg, asm.n_dofs, 2 * its


def assembly_cpu_baseline(n_sample: int, n_target: int):
    """The oracle's coupled solve plus an adjoint solve on two sizes,
    extrapolated to the workload as cpu_baseline does."""
    n_small = max(4, (2 * n_sample) // 3)
    t_s, cg_s, dofs_s, it_s = _assembly_port_step(n_small)
    t_l, cg_l, dofs_l, it_l = _assembly_port_step(n_sample)
    alpha = math.log(it_l / it_s) / math.log(n_sample / n_small) if it_s > 0 and it_l > 0 else 1.0
    dofs_t = 2 * 3 * (n_target + 1) ** 3 + 6
    it_t = it_l * (n_target / n_sample) ** alpha
    t_t = (t_l - cg_l) * (dofs_t / dofs_l) + cg_l * (dofs_t / dofs_l) * (it_t / it_l)
    return {"value": t_t / (dofs_t / 1e6), "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
            "sample": f"assembly oracle (numpy part matrices, T^T K T, scipy Jacobi-CG to 1e-10, solve + an "
                      f"adjoint solve of the same system) on the {n_small}^3 and {n_sample}^3 pairs ({dofs_s} and "
                      f"{dofs_l} DOF: {t_s:.2f} s and {t_l:.2f} s), extrapolated to {n_target}^3 ({dofs_t} DOF) "
                      f"with iterations ~ n^{alpha:.2f}",
            "samples": {"n": [n_small, n_sample], "seconds": [t_s, t_l], "cg_iterations": [it_s, it_l]}}


def run_assembly(args):
    """The assembly workload at n = --assembly-n: --warmup untimed and --steps
    timed coupled solves with the gradient, FP64 Jacobi CG on T^T K T (CUDA
    events); beside it the same box as one monolithic mesh in FP64."""
    from torchfem_gb300 import _lib

    dev = torch.device("cuda", 0)
    lib = _lib.load()
    n = args.assembly_n
    t0 = time.perf_counter()
    asm, a, E0, point = assembly_workload(n, dev)
    assembly_step(asm, a, E0, point, args.stol)
    torch.cuda.synchronize()
    first_ms = (time.perf_counter() - t0) * 1e3
    for _ in range(max(args.warmup, 0)):
        assembly_step(asm, a, E0, point, args.stol)
    stream = torch.cuda.current_stream(dev)
    lib.fem_set_timing(1)
    launches0 = lib.fem_launch_count()
    spmv_ms = spmv_n = 0
    iters = []
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clocks:
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(args.steps):
            u, g = assembly_step(asm, a, E0, point, args.stol)
            st = asm.last_solve
            iters.append(st.iterations)
            spmv_ms += st.spmv_ms
            spmv_n += st.spmv_timed
        ev1.record(stream)
        torch.cuda.synchronize()
    lib.fem_set_timing(0)
    launches = lib.fem_launch_count() - launches0
    ms = ev0.elapsed_time(ev1) / args.steps
    st = asm.last_solve
    n_dofs = asm.n_dofs
    peak, peak_kind = measured_peak_hbm()
    nr = st.n
    sb = st.nnz * 12 + (nr + 1) * 8 + 13 * 8 * nr  # FP64 CSR values + columns, row pointers, vector streams
    unit_s = spmv_ms / spmv_n / 1e3 if spmv_n else None
    achieved = sb / unit_s / 1e9 if unit_s else None
    # the same box as one mesh, FP64 Jacobi CG
    from torchfem_gb300 import Solid, mesh
    from torchfem_gb300.materials import IsotropicElasticity3D

    nodes, el = mesh.cube_hexa(2 * n + 1, n + 1, n + 1, 2.0, 1.0, 1.0)
    mono = Solid(nodes.to(dev), el.to(dev), IsotropicElasticity3D(1000.0, 0.3))
    mono.constraints[(nodes[:, 0] == 0.0).to(dev)] = True
    mono.forces[(nodes[:, 0] == 2.0).to(dev), 2] = 1.0 / int((nodes[:, 0] == 2.0).sum())
    fm = mono.forces.detach().clone().requires_grad_(True)

    def mono_step():
        mono.forces = fm
        uu, _, _, _, _ = mono.solve(stol=args.stol, differentiable_parameters=fm)
        torch.autograd.grad(uu.sum(), fm)

    mono_step()
    torch.cuda.synchronize()
    m0, m1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    m0.record(stream)
    mono_step()
    m1.record(stream)
    torch.cuda.synchronize()
    mono_ms = m0.elapsed_time(m1)
    line = {
        "metric": ASSEMBLY_METRIC, "value": ms / 1e3 / (n_dofs / 1e6), "unit": UNIT, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded jittered cubes)",
        "config": {"workload": f"assembly: two {n}^3 Hexa1 cubes tied at an interface, a reference point on the "
                               f"far face (moment + pull), work and d/dE of the first cube",
                   "dofs": n_dofs, "retained_dofs": nr, "coupled_nnz": st.nnz, "stol": args.stol},
        "cg_iterations": iters, "gpu_launches": launches,
        "setup_excluded_ms": {"models_pattern_and_first_solve": first_ms},
        "roofline": {"bound": "hbm", "kernel": "persistent FP64 Jacobi-CG kernel on T^T K T (one iteration)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None, "traffic": None, "algorithmic_bytes": sb,
                     "avg_unit_us": unit_s * 1e6 if unit_s else None, "peak_source": peak_kind},
        "monolithic_fp64": {"ms_per_step": mono_ms, "dofs": 3 * len(nodes),
                            "note": "the same 2 x 1 x 1 box as one unjittered mesh, FP64 Jacobi CG, solve + adjoint"},
        "clocks": clocks.summary(),
        "cpu_baseline": assembly_cpu_baseline(args.assembly_cpu_n, n),
    }
    print(json.dumps(line))


CONFIG_METRIC = "config {k}: solve+grad s per 1M DOF, mixed precision (FP32 multigrid CG + FP64 refinement) vs plain FP64"


def config_workload(k: int, device):
    """The benchmark configurations 3, 4 and 5 as (model, parameter, step):
    step(precision, precond) runs the configuration's solve and the gradient
    of its loss and returns (primary field, gradient).
      3: SIMP cantilever, Quad1 400 x 200, compliance f.u, dL/drho;
      4: Neo-Hookean Tetra2 box 30 x 10 x 10 pulled to +0.5 with nlgeom in 40
         increments (10 and 20 fail in the reference's algorithm as in this
         one), tip reaction, d/dE_e;
      5: J2 plane-strain O-grid plate 256 x 64 with a hole, 20 increments,
         reaction, d/d(thickness)."""
    from torchfem_gb300 import Planar, Solid, mesh
    from torchfem_gb300.materials import (Hyperelastic3D, IsotropicElasticityPlaneStress,
                                          IsotropicPlasticityPlaneStrain, neo_hookean_psi)

    if k == 3:
        nodes, el = mesh.rect_quad(401, 201, 2.0, 1.0)
        rho0 = 0.2 + 0.8 * torch.rand(len(el), generator=torch.Generator().manual_seed(0), dtype=torch.float64)
        tip = torch.argmin(((nodes - torch.tensor([2.0, 0.5])) ** 2).sum(1))

        def step(precision, precond):
            rho = rho0.to(device).requires_grad_(True)
            m = Planar(nodes.to(device), el.to(device), IsotropicElasticityPlaneStress(rho**3 * 1.0, 0.3))
            m.constraints[(nodes[:, 0] == 0.0).to(device), :] = True
            m.forces[tip, 1] = -1.0
            u, f, _, _, _ = m.solve(stol=1e-10, precision=precision, preconditioner=precond,
                                    differentiable_parameters=rho)
            (g,) = torch.autograd.grad(torch.inner(f.ravel(), u.ravel()), rho)
            return m, u, g
        return step, "quad1_simp_cantilever_400x200_compliance+dL/drho", {"stol": 1e-10}
    if k == 4:
        nodes, el = mesh.linear_to_quadratic(*mesh.box_tetra6(31, 11, 11, 3.0, 1.0, 1.0))
        E0 = 1000.0 * (1.0 + 0.1 * torch.randn(len(el), generator=torch.Generator().manual_seed(0),
                                               dtype=torch.float64))
        right = nodes[:, 0] == 3.0

        def step(precision, precond):
            E = E0.to(device).requires_grad_(True)
            nu = 0.45
            mu, lbd = E / (2.0 * (1.0 + nu)), E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))
            m = Solid(nodes.to(device), el.to(device), Hyperelastic3D(neo_hookean_psi, torch.stack([mu, lbd], -1)))
            m.constraints[(nodes[:, 0] == 0.0).to(device), :] = True
            m.constraints[right.to(device), 0] = True
            m.displacements[right.to(device), 0] = 0.5
            u, f, _, _, _ = m.solve(increments=torch.linspace(0.0, 1.0, 41), nlgeom=True, rtol=1e-10, atol=1e-10,
                                    max_iter=20, stol=1e-12, precision=precision, preconditioner=precond,
                                    differentiable_parameters=E)
            (g,) = torch.autograd.grad(f[right.to(device), 0].sum(), E)
            return m, u, g
        return step, "tetra2_neo_hookean_box_30x10x10_40_increments_reaction+dR/dE", \
            {"stol": 1e-12, "increments": 40, "newton_rtol": 1e-10}
    nodes, el = mesh.plate_hole_ogrid(256, 64)
    left = torch.isclose(nodes[:, 0], torch.tensor(0.0, dtype=torch.float64))
    right = torch.isclose(nodes[:, 0], torch.tensor(2.0, dtype=torch.float64))
    pin = torch.argmin(((nodes - torch.tensor([0.0, 0.5])) ** 2).sum(1))

    def step(precision, precond):
        mat = IsotropicPlasticityPlaneStrain(1000.0, 0.3, lambda q: 1.0 + 100.0 * q,
                                             lambda q: 100.0 * torch.ones_like(q))
        t = torch.ones(len(el), dtype=torch.float64, device=device, requires_grad=True)
        m = Planar(nodes.to(device), el.to(device), mat, thickness=t)
        m.constraints[left.to(device), 0] = True
        m.constraints[pin, 1] = True
        m.constraints[right.to(device), 0] = True
        m.displacements[right.to(device), 0] = 0.02
        u, f, _, _, _ = m.solve(increments=torch.linspace(0.0, 1.0, 21), rtol=1e-12, atol=1e-12, max_iter=80,
                                stol=1e-12, precision=precision, preconditioner=precond, differentiable_parameters=t)
        (g,) = torch.autograd.grad(f[right.to(device), 0].sum(), t)
        return m, u, g
    return step, "quad1_ogrid_plate_hole_256x64_j2_plane_strain_20_increments_reaction+dR/dt", \
        {"stol": 1e-12, "increments": 20, "newton_rtol": 1e-12}


def run_config(args):
    """One of the configurations 3, 4, 5 (--workload config3|config4|config5):
    --warmup untimed and --steps timed steps of the mixed path (multigrid),
    then one timed step of the FP64 path; CUDA events on the launching
    stream.  The roofline is the level-0 SpMV of the multigrid CG (its
    CUDA-event mean over the timed steps' last linear solve)."""
    from torchfem_gb300 import _lib

    k = int(args.workload[-1])
    dev = torch.device("cuda", 0)
    lib = _lib.load()
    stream = torch.cuda.current_stream(dev)
    stepf, name, settings = config_workload(k, dev)
    holder = {}

    def run(prec, pc):
        m, u, g = stepf(prec, pc)
        holder["m"] = m
        return (u, g), m

    for _ in range(max(args.warmup, 0)):
        run("mixed", "amg")
    torch.cuda.synchronize()
    ms, iters, u_ms, u_n, launches, clocks, (u_m, g_m) = timed_steps(lib, lambda: run("mixed", "amg"), args.steps,
                                                                     stream)
    m = holder["m"]
    dm = m.device_mesh
    n_dofs = m.n_dofs
    p_ms, p_iters, _, _, _, _, (u_p, g_p) = timed_steps(lib, lambda: run("fp64", None), 1, stream)
    peak, peak_kind = measured_peak_hbm()
    unit_s = (u_ms / u_n) / 1e3 if u_n else None
    sb = level0_launch_bytes(dm, args.smoother)
    achieved = sb / unit_s / 1e9 if unit_s else None
    line = {
        "metric": CONFIG_METRIC.format(k=k), "value": ms / 1e3 / (n_dofs / 1e6), "unit": UNIT, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic (seeded, the configuration's)",
        "config": {"workload": f"config{k}: {name}", "dofs": n_dofs, "nnz": dm.nnz, "n_elem": m.n_elem,
                   "preconditioner": "smoothed-aggregation multigrid", **settings},
        "cg_iterations_last_step": ({"solves": len(iters[-1]), "total": sum(iters[-1]),
                                     "max": max(iters[-1])} if iters and iters[-1] else None),
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "kernel": "k_sell_op<d,*> (level-0 SpMV of the multigrid CG)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None, "traffic": None, "algorithmic_bytes": sb,
                     "avg_unit_us": unit_s * 1e6 if unit_s else None, "peak_source": peak_kind},
        "plain_fp64": {"value": p_ms / 1e3 / (n_dofs / 1e6), "ms_per_step": p_ms},
        "mixed_speedup_vs_plain": p_ms / ms,
        "rel_err_mixed_vs_fp64": {"u": float((u_m - u_p).detach().abs().max() / u_p.detach().abs().max()),
                                  "grad": float((g_m - g_p).abs().max() / g_p.abs().max())},
        "clocks": clocks,
    }
    print(json.dumps(line))


def run_profile_step(args):
    """For a launch list: the cube's set-up, --warmup mixed steps, then
    exactly one more (the one a summary describes)."""
    dev = torch.device("cuda", 0)
    m, forces = cube_workload(args.n, dev)
    for _ in range(max(args.warmup, 0) + 1):
        step(m, forces, "mixed", args.stol, args.precond)
    torch.cuda.synchronize()
    print(json.dumps({"profile": "step", "n": args.n, "warmup": args.warmup, "preconditioner": args.precond,
                      "cg_iterations": m.last_solve.iterations}))


def run_profile(args):
    """A short, fixed launch sequence for ncu: setup, one assembly, then
    exactly --profile-iters CG iterations of the chosen precision."""
    from torchfem_gb300 import _lib

    dev = torch.device("cuda", 0)
    _lib.load().fem_set_cg_path({"persistent": 1, "persistent-regs": 2, "kernels": 0}[args.cg_path])
    m, forces = cube_workload(args.n, dev)
    dm = m.device_mesh
    kind, data = m.material.kernel_data(m.n_elem)
    data = data.to(dev).contiguous()
    mesh_s = dm.make_mesh(None)
    mat = _lib.FemMaterial(kind, data.data_ptr())
    con = m.constraints.reshape(-1).to(dev, torch.uint8).contiguous()
    sysm = dm.build_system(mesh_s, mat, con, args.profile, keep_refs=(data, mesh_s, mat),
                           precond=args.precond if args.profile == "mixed" else "jacobi")
    b = torch.where(con.bool(), torch.zeros_like(forces.reshape(-1)), forces.reshape(-1)).contiguous()
    try:
        dm.solve(sysm, b, 1e-30, max_iter=args.profile_iters)
    except RuntimeError:
        pass  # stopped by the iteration cap, as intended
    torch.cuda.synchronize()
    print(json.dumps({"profile": args.profile, "n": args.n, "iterations": sysm.stats.iterations,
                      "n_blocks": dm.n_blocks, "nnz": dm.nnz, "n_dofs": dm.n_dofs}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=70, help="elements per cube edge")
    ap.add_argument("--stol", type=float, default=1e-10)
    ap.add_argument("--cpu-n", type=int, default=24, help="cube size of the CPU baseline sample")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain FP64 comparison")
    ap.add_argument("--profile", choices=["mixed", "fp64", "step"], default=None,
                    help="profiling mode: assemble one system and run --profile-iters CG iterations "
                         "(mixed, fp64), or --warmup steps and then exactly one step (step)")
    ap.add_argument("--profile-iters", type=int, default=20)
    ap.add_argument("--cg-path", choices=["persistent", "persistent-regs", "kernels"], default="persistent")
    ap.add_argument("--precond", choices=["amg", "jacobi"], default="amg",
                    help="preconditioner of the mixed-precision headline")
    ap.add_argument("--workload", choices=["elastic", "heat", "thermal", "config3", "config4", "config5", "assembly"],
                    default="elastic")
    ap.add_argument("--amg-delta", type=float, default=None,
                    help="FP64 replacement threshold of the multigrid CG (default: the library's)")
    ap.add_argument("--smoother", choices=["fp16", "fp32"], default="fp16",
                    help="level-0 smoothing passes of the multigrid V-cycle: FP16 copy or the FP32 matrix")
    ap.add_argument("--pdl", type=int, choices=[0, 1], default=None,
                    help="programmatic dependent launch in the multigrid CG iteration (default: the library's)")
    ap.add_argument("--level0", choices=["ldg", "tma"], default="tma",
                    help="level-0 block SpMVs of the multigrid CG: direct loads, or slices streamed by bulk copies")
    ap.add_argument("--residual", choices=["auto", "copy", "elements"], default="auto",
                    help="FP64 residual of the mixed solvers: FP64 copy of the sliced matrix, the element pass, "
                         "or the library's choice (the copy for heat, the element pass for vector fields)")
    ap.add_argument("--thermal-n", type=int, default=1024, help="N of the thermal slab (N x N/2 x 1 elements)")
    ap.add_argument("--heat-n", type=int, default=100, help="elements per cube edge of the heat workload")
    ap.add_argument("--heat-cpu-n", type=int, default=30, help="cube size of the heat CPU baseline sample")
    ap.add_argument("--assembly-n", type=int, default=40, help="elements per cube edge of the assembly workload")
    ap.add_argument("--assembly-cpu-n", type=int, default=12, help="cube size of the assembly CPU baseline sample")
    args = ap.parse_args()
    torch.set_default_dtype(torch.float64)
    if args.impl == "reference":
        run_reference(args)
        return
    if torch.cuda.is_available():
        from torchfem_gb300 import _lib
        from torchfem_gb300.sparse import SolveContext

        from torchfem_gb300._device import LinearSystem

        _lib.load().fem_amg_set_half_smoother(1 if args.smoother == "fp16" else 0)
        _lib.load().fem_amg_set_level0_tma(1 if args.level0 == "tma" else 0)
        if args.pdl is not None:
            _lib.load().fem_amg_set_pdl(args.pdl)
        LinearSystem.RESIDUAL_COPY = {"auto": None, "copy": True, "elements": False}[args.residual]
        if args.amg_delta is not None:
            SolveContext.AMG_DELTA = args.amg_delta
    if args.workload.startswith("config"):
        run_config(args)
        return
    if args.workload == "heat":
        run_heat(args)
        return
    if args.workload == "assembly":
        run_assembly(args)
        return
    if args.workload == "thermal":
        run_thermal(args)
        return
    if args.profile == "step":
        run_profile_step(args)
        return
    if args.profile:
        run_profile(args)
        return

    dist, rank, world, local = dist_setup()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from torchfem_gb300 import _lib

    lib = _lib.load()
    lib.fem_set_cg_path({"persistent": 1, "persistent-regs": 2, "kernels": 0}[args.cg_path])
    m, forces = cube_workload(args.n, dev)
    # set-up kept out of the timed steps (once per mesh, and once per mesh and
    # constraint set): the pattern and geometry cache, and the symbolic
    # multigrid hierarchy (aggregation, tentative prolongator, patterns)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    dm = m.device_mesh
    torch.cuda.synchronize()
    setup_mesh_ms = (time.perf_counter() - t0) * 1e3
    n_dofs = m.n_dofs
    stream = torch.cuda.current_stream(dev)
    pc = args.precond
    amg_symbolic_ms = None
    if pc == "amg":
        con_mask = m.constraints.reshape(-1).to(dev).to(torch.uint8).contiguous()
        t0 = time.perf_counter()
        dm.amg_hierarchy(con_mask)
        torch.cuda.synchronize()
        amg_symbolic_ms = (time.perf_counter() - t0) * 1e3

    # warm-up (W untimed steps), then K timed steps of the mixed path
    for _ in range(max(args.warmup, 0)):
        out = step(m, forces, "mixed", args.stol, pc)
    torch.cuda.synchronize()
    lib.fem_set_timing(1)
    spmv_ms, spmv_n, iters = 0.0, 0, []
    launches0 = lib.fem_launch_count()
    if dist is not None:
        dist.barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clocks:
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(args.steps):
            out = step(m, forces, "mixed", args.stol, pc)
            st = m.last_solve
            iters.append(st.iterations)
            spmv_ms += st.system.stats.spmv_ms
            spmv_n += st.system.stats.spmv_timed
        ev1.record(stream)
        torch.cuda.synchronize()
    launches = lib.fem_launch_count() - launches0
    lib.fem_set_timing(0)
    ms = ev0.elapsed_time(ev1) / args.steps
    ms = reduce_max(dist, ms, dev)
    u_mixed, g_mixed = out[0], out[5]

    # end to end through the public API from host tensors
    m_host, forces_host = cube_workload(args.n, torch.device("cpu"))
    forces_host = forces_host.pin_memory()
    _ = m_host.device_mesh  # setup (pattern, geometry) outside the timed region
    e2e_out = step(m_host, forces_host, "mixed", args.stol, pc)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_out = step(m_host, forces_host, "mixed", args.stol, pc)
    torch.cuda.synchronize()
    e2e_ms = (time.perf_counter() - t0) * 1e3 / args.steps
    e2e_ms = reduce_max(dist, e2e_ms, dev)
    n_elem = m.n_elem
    h2d = 8 * n_dofs * 2 + n_dofs + 16 * n_elem  # forces, prescribed displacements, constraints, (lambda, G)
    d2h = sum(t.numel() * t.element_size() for t in e2e_out[:5]) + 8 * n_dofs  # outputs + gradient

    result = {}
    if not args.no_plain:
        out_p = step(m, forces, "fp64", args.stol)
        torch.cuda.synchronize()
        p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        p0.record(stream)
        out_p = step(m, forces, "fp64", args.stol)
        p1.record(stream)
        torch.cuda.synchronize()
        plain_ms = reduce_max(dist, p0.elapsed_time(p1), dev)
        u_p, g_p = out_p[0], out_p[5]
        err_u = float((u_mixed - u_p).abs().max() / u_p.abs().max())
        err_g = float((g_mixed - g_p).abs().max() / g_p.abs().max())
        err_s = float((out[2] - out_p[2]).abs().max() / out_p[2].abs().max())
        result = {"plain_fp64": {"value": plain_ms / 1e3 / (n_dofs / 1e6), "ms_per_step": plain_ms,
                                 "cg_iterations": m.last_solve.iterations},
                  "mixed_speedup_vs_plain": plain_ms / ms,
                  "rel_err_mixed_vs_fp64": {"u": err_u, "sigma": err_s, "grad": err_g}}
        if pc != "jacobi":
            # the mixed path with block Jacobi, same workload
            step(m, forces, "mixed", args.stol, "jacobi")
            torch.cuda.synchronize()
            j0, j1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            j0.record(stream)
            step(m, forces, "mixed", args.stol, "jacobi")
            j1.record(stream)
            torch.cuda.synchronize()
            bj_ms = reduce_max(dist, j0.elapsed_time(j1), dev)
            result["mixed_block_jacobi"] = {"value": bj_ms / 1e3 / (n_dofs / 1e6), "ms_per_step": bj_ms,
                                            "cg_iterations": m.last_solve.iterations,
                                            "speedup_vs_plain": plain_ms / bj_ms}

    peak, peak_kind = measured_peak_hbm()
    persistent = lib.fem_get_cg_path() in (1, 2) and pc == "jacobi"
    traffic = None
    if pc == "amg":
        # CUDA events around every level-0 SpMV launch of the multigrid CG
        # (four Chebyshev passes and q = A p per iteration)
        unit_s = (spmv_ms / spmv_n) / 1e3 if spmv_n else None
        sb = level0_launch_bytes(dm, args.smoother)
        kernel_name = ("k_sell_op<3,*> (level-0 block SpMV of the multigrid CG: four Chebyshev passes on the "
                       "%s matrix, q = A p on the FP32 matrix; fused epilogues)"
                       % ("FP16 smoothing copy of the" if args.smoother == "fp16" else "FP32"))
        traffic_file = ROOT / "profiles" / "amg_sell_op_traffic.json"
        if traffic_file.exists():
            try:
                traffic = json.loads(traffic_file.read_text())["dram_bytes_per_block_per_launch"] * dm.n_blocks
            except (KeyError, ValueError):
                traffic = None
    elif persistent:
        # CUDA events around each persistent CG launch; spmv_n counts the
        # iterations those launches ran
        unit_s = (spmv_ms / spmv_n) / 1e3 if spmv_n else None
        sb = cg_iteration_bytes(dm)
        kernel_name = "k_pcg_persistent<3,float,%d> (one CG iteration)" % (1 if lib.fem_get_cg_path() == 1 else 0)
    else:
        unit_s = (spmv_ms / spmv_n) / 1e3 if spmv_n else None
        sb = spmv_bytes(dm)
        kernel_name = "k_spmv_sell<3>"
    avg_spmv_s = unit_s
    achieved = sb / unit_s / 1e9 if unit_s else None
    # DRAM bytes per CG iteration from one ncu capture of the persistent kernel
    # (dram__bytes_read.sum + dram__bytes_write.sum over a 20-iteration launch),
    # per stored block so that it scales to this workload's matrix
    traffic_file = ROOT / "profiles" / "pcg_persistent_traffic.json"
    if persistent and traffic_file.exists():
        try:
            tj = json.loads(traffic_file.read_text())
            traffic = tj["dram_bytes_per_block_per_iteration"] * dm.n_blocks
        except (KeyError, ValueError):
            traffic = None

    if rank == 0:
        line = {
            "metric": METRIC,
            "value": ms / 1e3 / (n_dofs / 1e6),
            "unit": UNIT,
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": ms,
            "higher_is_better": False,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32+f64",
            "data": "synthetic (seeded jittered cube)",
            "config": {"workload": f"hexa1_cube_{args.n}^3_jittered_linear_elastic_solve+adjoint",
                       "preconditioner": "smoothed-aggregation multigrid" if pc == "amg" else "block Jacobi",
                       "level0_smoothing": args.smoother if pc == "amg" else None,
                       "fp64_residual": "FP64 copy of the sliced matrix" if args.residual == "copy"
                       else "element pass",
                       "dofs": n_dofs, "nnz": dm.nnz, "n_elem": n_elem, "stol": args.stol,
                       "parallelism": "replicas" if world > 1 else "single",
                       "l2": "inputs larger than L2 (FP32 K = %.0f MB)" % (dm.n_blocks * 40 / 1e6)},
            "cg_iterations": iters,
            "gpu_launches": launches,
            "setup_excluded_ms": {"mesh_pattern_and_geometry": setup_mesh_ms, "amg_symbolic": amg_symbolic_ms},
            "e2e": {"value": e2e_ms / 1e3 / (n_dofs / 1e6), "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms},
            "roofline": {"bound": "hbm", "kernel": kernel_name, "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": (achieved / peak) if achieved else None,
                         "traffic": traffic, "algorithmic_bytes": sb, "avg_unit_us": avg_spmv_s * 1e6 if avg_spmv_s else None,
                         "peak_source": peak_kind},
            "clocks": clocks.summary(),
            **result,
        }
        if world == 1:
            line["cpu_baseline"] = cpu_baseline(args.cpu_n, args.n)
        print(json.dumps(line))
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
