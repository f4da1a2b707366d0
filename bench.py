#!/usr/bin/env python
"""R+K assembly throughput on GB300 (Melem/s) with the HBM roofline of the
dominant kernel, for the 3D compressible Neo-Hookean workload: vector hex8 on a
128^3 structured box (2,097,152 elements, 6,440,067 dofs, 513,599,625 CSC
entries), 2x2x2 Gauss points, E = 1, nu = 0.3, displacement = affine stretch
diag(1.05, 0.98, 0.98) - I plus N(0, 1e-3^2) nodal noise (seed 1).

A step is one fused residual + tangent assembly (field update, element kernel,
deterministic node gather into the residual over unknowns and the CSC nzval).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload neohookean|poisson] [--precision fp64|fp32_element]

Under torchrun (N > 1) each rank assembles its own copy of the workload on its
own GPU (weak scaling, no collective on the data path); value = all ranks'
elements / max-over-ranks time.  --impl reference times the reference
algorithm's CPU implementation (element loop -> element-ordered COO ->
sparse!-style COO->CSC, OpenMP over the host cores) on a bounded sample of the
same workload; only rank 0 runs it.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
for _p in (str(ROOT / "finiteelementcontainers.jl_gb300"), str(ROOT)):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "R+K assembly Melem/s & % HBM roofline; MLP closure vs exact at 1e-3 stress err"
UNIT = "Melem/s"
# compulsory HBM bytes per element of one R+K pass (int32 connectivity, X and U
# gathers, residual and nzval written once)
WORKLOADS = {
    "neohookean": dict(n=128, kind="vector", name="neohookean_hex8_128cubed", flop_per_elem=48e3, state=0),
    "poisson": dict(n=32, kind="scalar", name="poisson_hex8_32cubed", flop_per_elem=8e3, state=0),
    # J2 plasticity: 8 points x 7 state values read (old) and written (new) per element
    "j2": dict(n=96, kind="vector", name="j2_hex8_96cubed", flop_per_elem=48e3, state=2 * 8 * 7 * 8),
    # J2 with the learned closure at plastic points, trained on 5M return-map samples (seed 4)
    "j2mlp": dict(n=96, kind="vector", name="j2_mlp_closure_hex8_96cubed", flop_per_elem=48e3,
                  state=2 * 8 * 7 * 8),
    # 64 uneven hex8 meshes (8^3..48^3, log-uniform, seed 2) in one block + a tet4/tet10/hex27 mesh,
    # a 5-iteration Newton-type loop replayed as one CUDA graph per step
    "batched": dict(n=0, kind="vector", name="batched_64_hex8_plus_tet4_tet10_hex27_newton5_graph",
                    flop_per_elem=48e3, state=0),
    # matrix-free tangent action K v of the Neo-Hookean 128^3 system (no K formed)
    "action": dict(n=128, kind="vector", name="neohookean_hex8_128cubed_matrix_free_action", flop_per_elem=5.5e3,
                   state=0),
    # the symbolic phase (CSC pattern + element maps) of the Neo-Hookean 128^3 system, host vs device
    "symbolic": dict(n=128, kind="vector", name="neohookean_hex8_128cubed_symbolic_phase", flop_per_elem=0,
                     state=0),
}
CPU_SAMPLE_N = {"neohookean": 40, "poisson": 32, "j2": 40, "batched": 40, "j2mlp": 40, "action": 40, "symbolic": 40}
J2_STEPS = 20
J2_PROPS = (200.0, 0.3, 0.25, 2.0)   # E, nu, yield stress, linear hardening


def algorithmic_bytes(ne: int, nn: int, nf: int, n_unknowns: int, nnz: int, nnpe: int = 8,
                      state_per_elem: int = 0) -> int:
    return 4 * nnpe * ne + 8 * 3 * nn + 8 * nf * nn + 8 * n_unknowns + 8 * nnz + state_per_elem * ne


def build_workload(fec, wl: str, n: int, device: int, precision: str, physics=None):
    """Mesh, assembler, parameters and the per-step inputs [(Uu, Dirichlet values or None)]."""
    from fec_gb300.workloads import stretch_field, uniaxial_bcs, uniaxial_inputs
    mesh = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (n + 1,) * 3)
    V = fec.FunctionSpace(mesh)
    if wl == "neohookean":
        var = fec.VectorFunction(V, "u")
        asm = fec.SparseMatrixAssembler(var, device=device, precision=precision)
        phys = fec.NeoHookean.from_youngs(1.0, 0.3)
        p = fec.create_parameters(mesh, asm, phys)
        U = stretch_field(mesh.nodal_coords, seed=1).ravel()
        inputs = [(np.ascontiguousarray(U[asm.dof.unknown_dofs - 1]), None)]
    elif wl == "j2":
        # symmetry on the x-, y-, z- faces, prescribed stretch on the x+ face; 20 load steps to 1% strain
        var = fec.VectorFunction(V, "u")
        asm = fec.SparseMatrixAssembler(var, device=device, precision=precision)
        phys = physics or fec.J2Plasticity(*J2_PROPS)
        p = fec.create_parameters(mesh, asm, phys, dirichlet_bcs=uniaxial_bcs())
        inputs = uniaxial_inputs(mesh.nodal_coords, asm.dof.unknown_dofs, p.bc_dofs.cpu().numpy(), J2_STEPS)
    else:
        var = fec.ScalarFunction(V, "u")
        asm = fec.SparseMatrixAssembler(var, device=device, precision=precision)
        bcs = [fec.DirichletBC("u", lambda X, t: 0.0, nodeset_name=f)
               for f in ("bottom", "right", "front", "top", "left", "back")]
        p = fec.create_parameters(mesh, asm, fec.Poisson(1.0), dirichlet_bcs=bcs)
        U = np.random.default_rng(0).uniform(-1.0, 1.0, mesh.num_nodes)
        inputs = [(np.ascontiguousarray(U[asm.dof.unknown_dofs - 1]), None)]
    asm._ensure_pattern()
    return mesh, asm, p, inputs


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        rows = []
        try:
            for line in Path(self.path).read_text().splitlines():
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9 and parts[1].replace(".", "").isdigit():
                    rows.append(parts)
        finally:
            try:
                os.unlink(self.path)
            except OSError:
                pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in rows]
        mx = max(float(r[2]) for r in rows)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        loaded = [s for s in sm if s > 0.5 * mx] or sm
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": mx, "reasons": reasons, "samples": len(rows),
                "power_w_max": max(float(r[3]) for r in rows if r[3].replace(".", "").isdigit())
                if any(r[3].replace(".", "").isdigit() for r in rows) else None}


def measured_peaks() -> dict:
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        d = json.loads(f.read_text())
        return {"hbm_gbs": d["hbm_gbs"], "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def profiled_traffic(workload: str) -> dict | None:
    """DRAM bytes per element of each kernel, from the committed ncu summary."""
    f = ROOT / "profiles" / f"traffic_{workload}.json"
    if f.exists():
        return json.loads(f.read_text())
    return None


def cpu_reference_run(wl: str, n: int, threads: int) -> tuple[float, int, str]:
    """One call of the reference algorithm on the host cores (oracle port):
    element loop (OpenMP, atomic residual scatter) + slot gather + sparse!.
    Returns (seconds, elements, description).  Pattern set-up is excluded, as
    the reference builds it once in update_dofs!."""
    from oracle import oracle
    from fec_gb300.workloads import stretch_field
    coords, conns = oracle.structured_hex8((n + 1,) * 3)
    nn = coords.shape[0]
    st_old = st_new = None
    if wl in ("neohookean", "batched"):
        nf, phys, props = 3, "neohookean", [1.0 / (3 * 0.4), 1.0 / 2.6]
        U = stretch_field(coords, seed=1).ravel()
        dd = np.zeros(0, dtype=np.int64)
    elif wl in ("j2", "j2mlp"):
        from fec_gb300.workloads import uniaxial_path
        nf, phys, props = 3, "j2", [200.0, 0.3, 0.25, 2.0]
        U = uniaxial_path(coords, J2_STEPS, nsteps=J2_STEPS, final_strain=0.01).ravel()
        dd = np.zeros(0, dtype=np.int64)
        st_old = np.zeros(7 * 8 * conns.shape[0])
        st_new = np.zeros_like(st_old)
    else:
        nf, phys, props = 1, "poisson", [1.0]
        U = np.random.default_rng(0).uniform(-1, 1, nn)
        dd = np.unique(np.concatenate([oracle.hex8_nodeset((n + 1,) * 3, f) for f in oracle.HEX8_FACES]))
    unknown, dtu = oracle.update_dofs(nf * nn, dd)
    blocks = [("HEX8", conns)]
    Is, Js, slots = oracle.pattern(blocks, nf, dtu)
    t0 = time.perf_counter()
    R, K = oracle.assemble(blocks, coords, phys, props, U, st_old, st_new, threads=threads)
    Ru = R[unknown - 1]
    oracle.sparse_csc(unknown.size, unknown.size, Is, Js, K[slots - 1])
    dt = time.perf_counter() - t0
    assert np.isfinite(Ru).all()
    return dt, conns.shape[0], f"{n}^3 hex8 {wl} (element loop on {threads} threads + serial sparse!)"


def cpu_baseline(wl: str, target_s: float = 10.0) -> dict:
    from oracle import oracle
    threads = oracle.max_threads()
    n = CPU_SAMPLE_N[wl]
    total, elems, reps = 0.0, 0, 0
    desc = ""
    while (total < target_s and reps < 5) or reps == 0:
        dt, ne, desc = cpu_reference_run(wl, n, threads)
        total += dt
        elems += ne
        reps += 1
    return {"value": elems / total / 1e6, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{reps} x {desc}, {total:.1f} s"}


def run_reference(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    if args.workload in ("action", "j2mlp", "batched", "symbolic"):
        print(json.dumps({"impl": "reference", "unavailable": f"the CPU port times the assembly workloads only "
                                                                f"(neohookean, poisson, j2), not {args.workload}"}))
        return
    from oracle import oracle
    threads = oracle.max_threads()
    n = CPU_SAMPLE_N[args.workload]
    for _ in range(args.warmup):
        cpu_reference_run(args.workload, n, threads)
    times, desc, ne = [], "", 0
    for _ in range(args.steps):
        dt, ne, desc = cpu_reference_run(args.workload, n, threads)
        times.append(dt)
    total = sum(times)
    value = ne * args.steps / total / 1e6
    wl = WORKLOADS[args.workload]
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": wl["name"], "precision": "fp64", "cpu_sample": f"{n}^3 elements per step"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{args.steps} x {desc}"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def exact_fp64_native_ms(args, n) -> float | None:
    """Milliseconds per load step of exact FP64 J2 assembly on the same path with
    the element contraction in native FP64 arithmetic (the selection is fixed per
    process, so it runs in a child process)."""
    env = dict(os.environ, FEC_FP64_CONTRACTION="native")
    cmd = [sys.executable, os.path.abspath(__file__), "--workload", "j2", "--n", str(n), "--steps", str(args.steps),
           "--warmup", str(args.warmup), "--no-cpu-baseline", "--no-e2e", "--no-variants"]
    r = subprocess.run(cmd, env=env, capture_output=True, text=True)
    if r.returncode != 0:
        return None
    try:
        return float(json.loads(r.stdout.strip().splitlines()[-1])["ms_per_step"])
    except (ValueError, KeyError, IndexError):
        return None


def run_closure(args) -> None:
    """Learned closure vs exact return mapping on the 96^3 J2 load path (20 steps,
    state carried), each path timed whole; errors per step against exact FP64."""
    import torch
    import __graft_entry__ as ge
    fec = ge.load_package()
    from fec_gb300 import closure
    torch.cuda.set_device(0)
    props = list(J2_PROPS)
    t0 = time.perf_counter()
    X, Y, plastic = closure.generate_samples(props, n_paths=args.paths, steps=20, seed=4)
    n_samples = int(X.shape[0])
    X, Y = X[plastic], Y[plastic]
    ntr = int(0.95 * X.shape[0])
    trained = closure.train(X[:ntr], Y[:ntr], epochs=args.epochs, batch=4096, lr=5e-3)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    val = closure.validation_errors(trained, props, X[ntr:], Y[ntr:])
    n = WORKLOADS["j2mlp"]["n"] if not args.n else args.n
    stream = torch.cuda.current_stream()

    def system(physics, precision):
        mesh, asm, p, inputs = build_workload(fec, "j2", n, 0, precision, physics=physics)
        dev = [(torch.from_numpy(u).cuda(), torch.from_numpy(b).cuda()) for u, b in inputs]
        return mesh, asm, p, dev

    launches = [0]

    def path(asm, p, dev, each=None):
        p.state_old.zero_()
        p.state_new.zero_()
        for i, (Uu, bc) in enumerate(dev):
            p.bc_vals = bc
            R, K = fec.assemble_residual_and_stiffness(asm, Uu, p)
            launches[0] += 2 + asm.last_launch_count()   # field update (Dirichlet + unknowns), elements, gather
            if each is not None:
                each(i, R, K, p)
            p.swap_states()

    def timed(asm, p, dev, stats=False):
        for _ in range(args.warmup):
            path(asm, p, dev)
        torch.cuda.synchronize()
        if stats:
            closure.J2Closure.stats(asm, reset=True)
        launches[0] = 0
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            path(asm, p, dev)
        e1.record(stream)
        torch.cuda.synchronize()
        per_step_launches[0] = launches[0] / (args.steps * J2_STEPS)
        return e0.elapsed_time(e1) / (args.steps * J2_STEPS)

    per_step_launches = [0]
    tols = (1e-4, 1e-3, 1e-2)
    mesh, a64, p64, d64 = system(None, "fp64")
    ne = mesh.num_elements()
    _, a32, p32, d32 = system(None, "fp32_element")
    cl = {}
    for tol in tols:
        phys = closure.J2Closure(*props, closure.TrainedClosure(trained.params, trained.normalisation, [], tol))
        cl[tol] = system(phys, "fp32_element")[1:]
    with ClockSampler(0) as clk:
        t_cl = {}
        for tol in tols:
            a, p, d = cl[tol]
            t_cl[tol] = timed(a, p, d, stats=True)
            if tol == tols[0]:
                main_launches = per_step_launches[0] * args.steps * J2_STEPS
        t_x32 = timed(a32, p32, d32)
        t_x64 = timed(a64, p64, d64)
    # per-step errors against exact FP64 (the paths run in lockstep)
    ref = []
    path(a64, p64, d64, lambda i, R, K, p: ref.append((R.clone(), K.nzval.clone(), p.state_new.clone())))

    def errors(asm, p, d):
        worst = {"residual": 0.0, "nzval": 0.0, "state": 0.0}

        def each(i, R, K, pp):
            Rr, Kr, Sr = ref[i]
            for k, a, b in (("residual", R, Rr), ("nzval", K.nzval, Kr), ("state", pp.state_new, Sr)):
                worst[k] = max(worst[k], float((a - b).norm() / b.norm()) if float(b.norm()) > 0 else 0.0)
        path(asm, p, d, each)
        return worst

    def kernels(asm, p, d):
        """Per-kernel milliseconds averaged over one path (CUDA events around each launch)."""
        acc: dict[str, list[float]] = {}
        asm.set_profiling(True)

        def each(i, R, K, pp):
            for name, ms in asm.kernel_times():
                acc.setdefault(name, []).append(ms)
        path(asm, p, d, each)
        asm.set_profiling(False)
        return {k: sum(v) / len(v) for k, v in acc.items()}

    out = {}
    for tol in tols:
        a, p, d = cl[tol]
        plast, fb = closure.J2Closure.stats(a, reset=True)   # over the timed repetitions
        calls = args.steps * J2_STEPS
        err = errors(a, p, d)
        out[f"tol_{tol:g}"] = {
            "ms_per_load_step": t_cl[tol], "Melem_per_s": ne / (t_cl[tol] * 1e-3) / 1e6,
            "plastic_points_per_path": plast * J2_STEPS // calls, "fallback_rate": fb / max(plast, 1),
            "max_rel_err_vs_exact_fp64_over_path": err, "kernels_ms": kernels(a, p, d)}
    x32_err = errors(a32, p32, d32)
    x_kernels = {"fp32_element": kernels(a32, p32, d32), "fp64": kernels(a64, p64, d64)}
    t_x64n = exact_fp64_native_ms(args, n)
    main_t = t_cl[1e-4]
    line = {
        "metric": METRIC, "value": ne / (main_t * 1e-3) / 1e6, "unit": UNIT, "n_gpus": 1,
        "steps": args.steps * J2_STEPS, "warmup": args.warmup * J2_STEPS, "ms_per_step": main_t,
        "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32-element (bf16 closure weights)", "data": "synthetic",
        "config": {"workload": WORKLOADS["j2mlp"]["name"], "elements": ne,
                   "step": f"one load step of the {J2_STEPS}-step uniaxial path (R+K, state carried); "
                           f"the timed region runs the whole path {args.steps} times",
                   "network": "14-64-64-64-64-13 SiLU, BF16 weights, FP32 accumulation",
                   "training": {"samples_generated": n_samples, "plastic_samples_used": int(ntr),
                                "epochs": args.epochs, "seconds": round(t_train, 1),
                                "final_loss": trained.history[-1]},
                   "l2": "inputs larger than L2"},
        "closure": {"validation_rel_err": val, **out},
        "exact": {"fp32_element_ms_per_load_step": t_x32, "fp64_ms_per_load_step": t_x64,
                  "fp32_element_max_rel_err_vs_fp64": x32_err, "kernels_ms": x_kernels,
                  "fp64_native_ms_per_load_step": t_x64n,
                  "fp64_native": "exact FP64 assembly with every product in native FP64 arithmetic "
                                 "(the reference's arithmetic; FEC_FP64_CONTRACTION=native), same path",
                  "speedup_closure_vs_exact_fp64": t_x64 / main_t, "speedup_closure_vs_exact_fp32": t_x32 / main_t,
                  "speedup_closure_vs_exact_fp64_native": (t_x64n / main_t) if t_x64n else None},
        "clocks": clk.summary(), "e2e": None, "gpu_launches": int(main_launches), "cpu_baseline": None,
    }
    print(json.dumps(line), flush=True)


def run_symbolic(args) -> None:
    """The symbolic phase of the Neo-Hookean 128^3 system (no Dirichlet dofs): CSC
    pattern, node adjacency, neighbour lists, column offsets and the element map,
    built by the host threads (fec_pattern_build) and by kernels
    (fec_pattern_build_device); each timed from the call to its return."""
    import ctypes as C
    import torch
    import __graft_entry__ as ge
    fec = ge.load_package()
    torch.cuda.set_device(0)
    n = args.n or WORKLOADS["symbolic"]["n"]
    mesh, asm, p, inputs = build_workload(fec, "neohookean", n, 0, "fp64")
    lib = fec.load_library()
    ctx = asm._ctx
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    nnz = C.c_int64()

    def host():
        assert lib.fec_pattern_build(ctx, C.byref(nnz)) == 0
        return int(nnz.value)

    def device():
        assert lib.fec_pattern_build_device(ctx, C.byref(nnz), s) == 0
        return int(nnz.value)

    times = {}
    sizes = {}
    for name, fn in (("host", host), ("device", device)):
        for _ in range(max(1, args.warmup)):
            sizes[name] = fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            fn()
        torch.cuda.synchronize()
        times[name] = (time.perf_counter() - t0) / args.steps
    assert sizes["host"] == sizes["device"]
    cores = os.cpu_count() or 1
    line = {"metric": "symbolic phase seconds (CSC pattern + element maps)", "value": times["device"], "unit": "s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": times["device"] * 1e3,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "int64", "data": "synthetic",
            "config": {"workload": WORKLOADS["symbolic"]["name"], "elements": mesh.num_elements(),
                       "nodes": mesh.num_nodes, "nnz": sizes["device"]},
            "host_threads_s": times["host"], "host_threads": cores, "speedup_device_vs_host": times["host"] / times["device"],
            "e2e": None, "gpu_launches": None, "cpu_baseline": None}
    print(json.dumps(line), flush=True)


def run_action(args) -> None:
    """Matrix-free tangent action of the Neo-Hookean 128^3 system: one step is
    field update + element action kernel + node gather (K v over the unknowns)."""
    import torch
    import __graft_entry__ as ge
    fec = ge.load_package()
    torch.cuda.set_device(0)
    n = args.n or WORKLOADS["action"]["n"]
    mesh, asm, p, inputs = build_workload(fec, "neohookean", n, 0, args.precision)
    ne, nn = mesh.num_elements(), mesh.num_nodes
    n_u = int(asm.dof.unknown_dofs.size)
    Uu = torch.from_numpy(inputs[0][0]).cuda()
    Vu = torch.from_numpy(np.random.default_rng(4).standard_normal(n_u)).cuda()
    stream = torch.cuda.current_stream()

    def step(u=Uu, v=Vu):
        return fec.assemble_matrix_free_action(asm, fec.stiffness_action, u, v, p)

    for _ in range(max(args.warmup, 3)):
        step()
    asm.set_profiling(True)
    step()
    kernels = {k: ms for k, ms in asm.kernel_times()}
    asm.set_profiling(False)
    torch.cuda.synchronize()
    with ClockSampler(0) as clk:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
    t_ms = e0.elapsed_time(e1) / args.steps
    # end to end: host Uu, Vu in (pinned), K v out (pinned)
    hU, hV = Uu.cpu().pin_memory(), Vu.cpu().pin_memory()
    hK = torch.empty(n_u, dtype=torch.float64).pin_memory()
    for _ in range(2):
        step(hU.cuda(non_blocking=True), hV.cuda(non_blocking=True))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        kv = step(hU.cuda(non_blocking=True), hV.cuda(non_blocking=True))
        hK.copy_(kv, non_blocking=True)
    torch.cuda.synchronize()
    t_e2e = (time.perf_counter() - t0) / args.steps
    # compulsory traffic: connectivity, X, U and V per node, K v over the unknowns
    alg = 4 * 8 * ne + 8 * 3 * nn * 3 + 8 * n_u
    dom = max((k for k in kernels if k != "update_field"), key=kernels.get)
    peaks = measured_peaks()
    achieved = alg / (t_ms * 1e-3) / 1e9
    line = {
        "metric": METRIC, "value": ne / (t_ms * 1e-3) / 1e6, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32-element/f64-accumulate",
        "data": "synthetic",
        "config": {"workload": WORKLOADS["action"]["name"], "elements": ne, "unknowns": n_u,
                   "precision": args.precision, "direction": "N(0,1) seed 4",
                   "l2": "inputs larger than L2 (X, U, V 155 MB; element workspace 403 MB)"},
        "roofline": {"bound": "hbm", "kernel": "whole step", "achieved": achieved, "peak": peaks["hbm_gbs"],
                     "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"], "traffic": None,
                     "algorithmic_bytes_per_elem": alg / ne, "kernels_ms": kernels, "dominant": dom},
        "e2e": {"value": ne / t_e2e / 1e6, "unit": UNIT, "h2d_bytes_per_step": 16 * n_u,
                "d2h_bytes_per_step": 8 * n_u},
        "clocks": clk.summary(), "gpu_launches": int(asm.last_launch_count() + 2) * args.steps,
        "cpu_baseline": None,
    }
    print(json.dumps(line), flush=True)


def run_batched(args) -> None:
    """The batched workload: both systems assembled 5 times per step inside one CUDA graph."""
    import torch
    import __graft_entry__ as ge
    fec = ge.load_package()
    from fec_gb300 import batching
    from fec_gb300.workloads import stretch_field
    torch.cuda.set_device(0)
    if args.n:  # reduced case (profiling): 8 meshes and an n^3-box mixed mesh
        meshes = {"batch8": batching.box_batch(batching.lognormal_cube_sides(count=8)).mesh,
                  "tet4_tet10_hex27": batching.mixed_mesh(args.n, args.n, args.n)}
    else:
        meshes = {"batch64": batching.box_batch(batching.lognormal_cube_sides()).mesh,
                  "tet4_tet10_hex27": batching.mixed_mesh(32, 32, 46)}
    phys = fec.NeoHookean.from_youngs(1.0, 0.3)
    systems, info = [], {}
    total_ne, alg = 0, 0
    for name, mesh in meshes.items():
        asm = fec.SparseMatrixAssembler(fec.VectorFunction(fec.FunctionSpace(mesh), "u"), device=0,
                                        precision=args.precision)
        p = fec.create_parameters(mesh, asm, phys)
        if args.single_launch:
            asm.set_single_launch(True)
        U = stretch_field(mesh.nodal_coords, seed=2).ravel()
        Uu = torch.from_numpy(U[asm.dof.unknown_dofs - 1].copy()).cuda()
        asm._ensure_pattern()
        systems.append((asm, p, Uu))
        ne = mesh.num_elements()
        nnpe = sum(mesh.element_conns[b].size for b in mesh.element_block_names) / ne
        total_ne += ne
        alg += algorithmic_bytes(ne, mesh.num_nodes, 3, int(asm.dof.unknown_dofs.size), asm.nnz, nnpe=nnpe)
        info[name] = {"elements": ne, "blocks": {b: (mesh.element_types[b], int(mesh.element_conns[b].shape[0]))
                                                 for b in mesh.element_block_names}, "nnz": asm.nnz}
    iters = 5
    loop = batching.NewtonLoop(systems, iterations=iters).capture()
    # eager reference timing of the same loop and per-kernel times (CUDA events on the launching stream)
    eager = batching.NewtonLoop(systems, iterations=iters)
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        eager.run_eager()
        loop.replay()
    torch.cuda.synchronize()
    a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a0.record(stream)
    for _ in range(args.steps):
        eager.run_eager()
    a1.record(stream)
    torch.cuda.synchronize()
    t_eager = a0.elapsed_time(a1)
    per_kernel: dict[str, list[float]] = {}
    for asm, p, Uu in systems:
        asm.set_profiling(True)
        fec.assemble_residual_and_stiffness(asm, Uu, p)
        for k, ms in asm.kernel_times():
            per_kernel.setdefault(k, []).append(ms)
        asm.set_profiling(False)
    torch.cuda.synchronize()
    with ClockSampler(0) as clk:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            loop.replay()
        e1.record(stream)
        torch.cuda.synchronize()
    t_ms = e0.elapsed_time(e1)
    value = iters * total_ne * args.steps / (t_ms * 1e-3) / 1e6
    kern_ms = {k: sum(v) for k, v in per_kernel.items()}
    dom = max(kern_ms, key=kern_ms.get)
    peaks = measured_peaks()
    step_ms = sum(kern_ms.values())
    single = bool(args.single_launch and args.precision == "fp64")
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "f32-element/f64-accumulate", "data": "synthetic",
        "config": {"workload": WORKLOADS["batched"]["name"], "elements": total_ne, "systems": info,
                   "newton_iterations": iters, "execution": "one CUDA graph replay per step",
                   "element_launches": ("one persistent launch per system for all its element blocks"
                                        if single else "one launch per element block"),
                   "autotune": fec.autotune_report(),
                   "precision": args.precision, "l2": "inputs larger than L2"},
        "eager_ms_per_step": t_eager / args.steps,
        "roofline": {"bound": "hbm", "kernel": "all kernels of one R+K pass of both systems",
                     "achieved": alg / (step_ms * 1e-3) / 1e9, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": alg / (step_ms * 1e-3) / 1e9 / peaks["hbm_gbs"], "traffic": None,
                     "kernels_ms_one_pass": kern_ms, "dominant": dom},
        "clocks": clk.summary(), "e2e": None,
        "gpu_launches": int(iters * sum(2 + (1 if single else len(a.fspace.block_names)) for a, _, _ in systems)
                            * args.steps),
        "cpu_baseline": None,
    }
    print(json.dumps(line), flush=True)


def run_ours(args) -> None:
    import torch
    import torch.distributed as dist
    import __graft_entry__ as ge
    fec = ge.load_package()

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl", device_id=torch.device(f"cuda:{local}"))
    torch.cuda.set_device(local)
    wl = dict(WORKLOADS[args.workload])
    if args.n:
        wl["n"] = args.n
        wl["name"] = wl["name"].split("_")[0] + f"_hex8_{args.n}cubed"
    mesh, asm, p, inputs = build_workload(fec, args.workload, wl["n"], local, args.precision)
    ne, nn, nf = mesh.num_elements(), mesh.num_nodes, asm.dof.nf
    n_u = int(asm.dof.unknown_dofs.size)
    stream = torch.cuda.current_stream()
    dev_inputs = [(torch.from_numpy(u).cuda(), None if b is None else torch.from_numpy(b).cuda()) for u, b in inputs]
    stateful = any(ph.NS for ph in p.physics)
    counter = [0]

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    def step(precision=None, feed=None, out=None):
        """One load step: Dirichlet values and unknowns of step i, fused R+K, state swap."""
        i = counter[0] % len(inputs)
        counter[0] += 1
        Uu, bc = (feed or dev_inputs)[i]
        if bc is not None:
            p.bc_vals = bc if bc.is_cuda else bc.to(asm._torch_device(), non_blocking=True)
        R, K = fec.assemble_residual_and_stiffness(asm, Uu, p, precision=precision, out=out)
        if stateful:
            p.swap_states()
        return R, K

    # ---- device-resident timing -------------------------------------------------
    for _ in range(args.warmup):
        step()
    asm.set_profiling(True)
    per_kernel: dict[str, list[float]] = {}
    launches = 0
    barrier()
    with ClockSampler(local) as clk:
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            step()
            for name, ms in asm.kernel_times():
                per_kernel.setdefault(name, []).append(ms)
                launches += 1
        e1.record(stream)
        barrier()
    asm.set_profiling(False)
    t_ms = e0.elapsed_time(e1)
    if world > 1:
        tt = torch.tensor([t_ms], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_ms = float(tt.item())
    clocks = clk.summary()
    value = world * ne * args.steps / (t_ms * 1e-3) / 1e6

    # ---- the other precision variant, same inputs --------------------------------
    variants = {}
    R0, K0 = step()
    nnz = K0.nnz
    if not args.no_variants:
        other = "fp32_element" if args.precision == "fp64" else "fp64"
        if not stateful:  # compare the two variants on identical inputs
            ref_R, ref_nz = R0.clone(), K0.nzval.clone()
        for _ in range(args.warmup):
            step(other)
        asm.set_profiling(True)
        vk: dict[str, list[float]] = {}
        barrier()
        g0 = torch.cuda.Event(enable_timing=True)
        g1 = torch.cuda.Event(enable_timing=True)
        g0.record(stream)
        for _ in range(args.steps):
            Rv, Kv = step(other)
            for name, ms in asm.kernel_times():
                vk.setdefault(name, []).append(ms)
        g1.record(stream)
        barrier()
        asm.set_profiling(False)
        tv = g0.elapsed_time(g1)
        variants[other] = {
            "value": world * ne * args.steps / (tv * 1e-3) / 1e6, "ms_per_step": tv / args.steps,
            "kernels_ms": {k: sum(v) / len(v) for k, v in vk.items()}}
        if not stateful:
            variants[other]["rel_err_vs_" + args.precision] = {
                "nzval": float((Kv.nzval - ref_nz).norm() / ref_nz.norm()),
                "residual": float((Rv - ref_R).norm() / ref_R.norm())}
            del ref_R, ref_nz
        R0, K0 = step()
    stateful_errors = None
    if stateful and not args.no_variants:
        stateful_errors = path_errors(fec, asm, p, dev_inputs, args.precision,
                                      "fp32_element" if args.precision == "fp64" else "fp64")
    if args.no_e2e:
        return finish(args, fec, world, rank, local, wl, mesh, asm, ne, nn, nf, n_u, nnz, t_ms, value, clocks,
                      per_kernel, launches, None, variants, stateful_errors)
    host_inputs = [(torch.from_numpy(u).pin_memory(), None if b is None else torch.from_numpy(b).pin_memory())
                   for u, b in inputs]
    n_bc = 0 if inputs[0][1] is None else int(inputs[0][1].size)
    R_h = torch.empty(n_u, dtype=torch.float64).pin_memory()
    nz_h = torch.empty(nnz, dtype=torch.float64).pin_memory()
    # Pipelined read-back: the steps write two output pairs in turn (the public call's
    # out= buffers) and each pair is read back on a copy stream while the next step
    # assembles into the other; every step's read-back is inside the timed region (the
    # region ends after the last one).
    copy_stream = torch.cuda.Stream()
    pairs = [(torch.empty(n_u, dtype=torch.float64, device=stream.device),
              torch.empty(nnz, dtype=torch.float64, device=stream.device)) for _ in range(2)]
    read_done = [torch.cuda.Event(), torch.cuda.Event()]
    for ev in read_done:
        ev.record(copy_stream)
    turn = [0]

    def e2e_step():
        j = turn[0] & 1
        turn[0] += 1
        stream.wait_event(read_done[j])          # the read-back two steps ago has left pair j
        R, K = step(feed=host_inputs, out=pairs[j])
        done = torch.cuda.Event()
        done.record(stream)
        copy_stream.wait_event(done)
        with torch.cuda.stream(copy_stream):
            R_h.copy_(R, non_blocking=True)
            nz_h.copy_(K.nzval, non_blocking=True)
        read_done[j].record(copy_stream)

    for _ in range(max(1, args.warmup)):
        e2e_step()
    for ev in read_done:
        stream.wait_event(ev)
    barrier()
    f0 = torch.cuda.Event(enable_timing=True)
    f1 = torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    for _ in range(args.steps):
        e2e_step()
    for ev in read_done:
        stream.wait_event(ev)
    f1.record(stream)
    barrier()
    t_e2e = f0.elapsed_time(f1)
    if world > 1:
        tt = torch.tensor([t_e2e], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_e2e = float(tt.item())
    e2e_value = world * ne * args.steps / (t_e2e * 1e-3) / 1e6
    e2e = {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 8 * (n_u + n_bc),
           "d2h_bytes_per_step": 8 * (n_u + nnz),
           "pipelining": "two output pairs in turn: the read-back of step i (copy stream) overlaps the assembly "
                         "of step i+1 into the other pair"}
    finish(args, fec, world, rank, local, wl, mesh, asm, ne, nn, nf, n_u, nnz, t_ms, value, clocks, per_kernel,
           launches, e2e, variants, stateful_errors)


def path_errors(fec, asm, p, dev_inputs, main: str, other: str) -> dict:
    """One clean pass of a stateful load path (state from zero) in both precisions
    in lockstep, each carrying its own state: the worst relative error (2-norm)
    of the `other` variant against `main` over the path, per output."""
    import torch
    saved = (p.state_old, p.state_new)
    s_main = [torch.zeros_like(p.state_old), torch.zeros_like(p.state_old)]
    s_oth = [torch.zeros_like(p.state_old), torch.zeros_like(p.state_old)]
    worst = {"residual": 0.0, "nzval": 0.0, "state": 0.0}
    for Uu, bc in dev_inputs:
        p.bc_vals = bc
        p.state_old, p.state_new = s_main
        R, K = fec.assemble_residual_and_stiffness(asm, Uu, p, precision=main)
        Rr, Kr = R.clone(), K.nzval.clone()
        p.state_old, p.state_new = s_oth
        R2, K2 = fec.assemble_residual_and_stiffness(asm, Uu, p, precision=other)
        for k, a, b in (("residual", R2, Rr), ("nzval", K2.nzval, Kr), ("state", s_oth[1], s_main[1])):
            nb = float(b.norm())
            if nb > 0:
                worst[k] = max(worst[k], float((a - b).norm()) / nb)
        del Rr, Kr
        s_main.reverse()
        s_oth.reverse()
    p.state_old, p.state_new = saved
    return {f"{other}_vs_{main}_max_rel_err_over_path": worst}


def finish(args, fec, world, rank, local, wl, mesh, asm, ne, nn, nf, n_u, nnz, t_ms, value, clocks, per_kernel,
           launches, e2e, variants, stateful_errors=None):
    import torch.distributed as dist
    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return

    # ---- roofline of the dominant kernel ------------------------------------------
    peaks = measured_peaks()
    totals = {k: sum(v) for k, v in per_kernel.items()}
    dom = max(totals, key=totals.get)
    avg_ms = totals[dom] / len(per_kernel[dom])
    alg_bytes = algorithmic_bytes(ne, nn, nf, n_u, nnz, state_per_elem=wl["state"])
    achieved = alg_bytes / (avg_ms * 1e-3) / 1e9
    traffic = None
    prof = profiled_traffic(wl["name"] + "_" + args.precision)
    if prof and dom in prof.get("bytes_per_elem", {}):
        traffic = prof["bytes_per_elem"][dom] * ne
    roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / peaks["hbm_gbs"], "peak_source": peaks["source"] + " (burst copy)",
                "traffic": traffic, "algorithmic_bytes_per_elem": alg_bytes / ne,
                "kernels_ms": {k: sum(v) / len(v) for k, v in per_kernel.items()},
                "kernel_share": {k: v / sum(totals.values()) for k, v in totals.items()}}
    fp = {}
    lib = fec.load_library()
    import ctypes as C
    for prec, code in (("fp64", 0), ("fp32", 1)):
        tf = C.c_double()
        if lib.fec_probe_fma_rate(local, code, C.byref(tf)) == 0:
            fp[prec] = tf.value
    elem_ms = sum(v for k, v in roofline["kernels_ms"].items() if k.startswith("element"))
    pipe = "fp64" if args.precision == "fp64" else "fp32"
    compute = {"pipe": pipe, "flop_per_elem": wl["flop_per_elem"],
               "achieved_tflops": wl["flop_per_elem"] * ne / (elem_ms * 1e-3) / 1e12,
               "peak_tflops": fp.get(pipe), "peak_source": "measured FMA probe (fec_probe_fma_rate)"}
    if compute["peak_tflops"]:
        compute["frac"] = compute["achieved_tflops"] / compute["peak_tflops"]
    if args.precision == "fp64" and args.workload == "neohookean":
        compute["note"] = ("FP64 results; the hex8 tangent contraction runs in double-float (df64) arithmetic on the "
                           "FP32 pipes, so the FP64-equivalent rate can exceed the native FP64 FMA peak "
                           f"({fp.get('fp32', 0):.1f} TFLOP/s FP32 measured)")

    cpu = None
    if world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(args.workload)
    if stateful_errors is not None:
        variants.setdefault("path_errors", stateful_errors)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32-element/f64-accumulate",
        "data": "synthetic",
        "config": {"workload": wl["name"], "elements": ne, "dofs": nf * nn, "nnz": nnz, "precision": args.precision,
                   **({"load_path": f"{J2_STEPS} uniaxial steps to 1% strain, state carried"} if wl["state"] else {}),
                   "quadrature": "2x2x2 Gauss", "l2": "inputs larger than L2 (element scratch %.1f GB, nzval %.1f GB)"
                   % ((ne * (nf * 8) ** 2 * (8 if args.precision == "fp64" else 4)) / 1e9, nnz * 8 / 1e9),
                   "parallelism": f"{world} independent replicas" if world > 1 else "single GPU"},
        "roofline": roofline,
        "compute_roofline": compute,
        "clocks": clocks,
        "e2e": e2e,
        "gpu_launches": launches,
        "cpu_baseline": cpu,
        "variants": variants,
    }
    if world == 1 and args.workload == "neohookean" and not args.no_sub_results:
        line["sub_results"] = sub_results(args)
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


# The other workloads, each run as its own process after the headline one and
# reported inside the headline line.  (steps, warmup) are capped so that the
# whole default run stays within a few minutes; the closure run trains its
# network first (5M return-map samples, 60 epochs).
SUB_RESULTS = (
    ("poisson_hex8_32cubed", ["--workload", "poisson"], None),
    ("j2_hex8_96cubed_20_step_path", ["--workload", "j2"], None),
    ("j2_mlp_closure_hex8_96cubed", ["--workload", "j2mlp"], (2, 1)),
    ("batched_64_hex8_plus_tet4_tet10_hex27", ["--workload", "batched"], (5, 2)),
    ("matrix_free_action_neohookean_128cubed", ["--workload", "action"], None),
    ("symbolic_phase_neohookean_128cubed", ["--workload", "symbolic"], (3, 1)),
)


def sub_results(args) -> dict:
    out = {}
    for name, extra, cap in SUB_RESULTS:
        steps, warmup = (min(args.steps, cap[0]), min(args.warmup, cap[1])) if cap else (args.steps, args.warmup)
        cmd = [sys.executable, os.path.abspath(__file__), *extra, "--steps", str(steps), "--warmup", str(warmup),
               "--no-sub-results"]
        t0 = time.perf_counter()
        try:
            r = subprocess.run(cmd, capture_output=True, text=True, timeout=900)
            lines = [ln for ln in r.stdout.strip().splitlines() if ln.startswith("{")]
            if r.returncode == 0 and lines:
                out[name] = json.loads(lines[-1])
            else:
                out[name] = {"error": f"exit {r.returncode}: {(r.stderr or r.stdout)[-400:]}"}
        except subprocess.TimeoutExpired:
            out[name] = {"error": "timed out after 900 s"}
        out[name]["wall_s"] = round(time.perf_counter() - t0, 1)
    return out


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="neohookean")
    ap.add_argument("--precision", choices=["fp64", "fp32_element"], default="fp64")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end (host buffer) measurement")
    ap.add_argument("--n", type=int, default=None, help="elements per box side (default: the workload's size)")
    ap.add_argument("--no-variants", action="store_true", help="skip timing the other precision variant")
    ap.add_argument("--no-sub-results", action="store_true",
                    help="default workload only: skip running the other workloads as sub-results")
    ap.add_argument("--single-launch", action="store_true",
                    help="batched FP64: every element block of a system in one persistent launch")
    ap.add_argument("--epochs", type=int, default=60, help="closure training epochs (j2mlp workload)")
    ap.add_argument("--paths", type=int, default=250_000,
                    help="random strain paths of 20 steps for the closure's training data (j2mlp workload)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batched":
        run_batched(args)
    elif args.workload == "j2mlp":
        run_closure(args)
    elif args.workload == "action":
        run_action(args)
    elif args.workload == "symbolic":
        run_symbolic(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
