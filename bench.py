"""Benchmark: finite-elasticity assembly throughput (elements/s) on one GB300.

Workload (default): the single-large-mesh configuration — a 32x32x32 box of
triquadratic Lagrange displacement / trilinear pressure elements (274,625 u
nodes, 859,812 dofs, 178,723,696 Jacobian nonzeros) with interior nodes
perturbed by seeded +-0.1h noise, incompressible Mooney-Rivlin c1=2, c2=6.
One step = one assembly of the mixed-precision Jacobian (FP32 uu block, FP64
coupling) together with the FP64 residual, at a seeded deformed state (stretch
1.1, shear 0.05).  All inputs are synthetic; the reference has no dataset for
this path.

value       elements/s with x resident in device memory (CUDA events around K
            steps on the launching stream);
e2e         the same through the C ABI with host (pinned) buffers: the dof
            vector is copied in and the assembled Jacobian + residual copied
            out every step;
roofline    algorithmic bytes of one assembly / its duration, against the
            measured HBM copy bandwidth;
cpu_baseline the FP64 CPU oracle (a restatement of the reference's Fortran
            assembly) on this host's cores, on a bounded sample.

--impl reference runs that CPU restatement alone (all host threads) on the
same workload and prints the same metric.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "assembled elements/s (Jacobian+residual)"
UNIT = "elements/s"


def config_mesh(name):
    from cm_gb300 import mesh as M
    if name == "cfg2":
        m = M.regular_box(32, 32, 32, nxi_u=3, pressure="node", law=M.MR, materials=(2.0, 6.0),
                          perturb=0.1, seed=2)
        workload = ("32x32x32 triquadratic-u/trilinear-p box, MR c1=2 c2=6, interior nodes +-0.1h, "
                    "mixed-precision Jacobian + FP64 residual")
    elif name == "cfg4":
        m = M.regular_box(16, 16, 16, nxi_u=3, pressure="node", law=M.MR, materials=(2.0, 6.0))
        workload = ("16x16x16 triquadratic-u/trilinear-p unit cube, MR c1=2 c2=6, "
                    "mixed-precision Jacobian + FP64 residual")
    elif name == "cfg5":
        m = M.guccione_slab(64, 64, 16, seed=0)
        workload = ("64x64x16 triquadratic-u/trilinear-p slab 40x40x10 mm, Guccione C=0.88 bf=18.5 bt=3.58 "
                    "bfs=1.63, fibre angle -60..+60 deg through the thickness +-5 deg noise, 2 kPa on z=0, "
                    "mixed-precision Jacobian + FP64 residual")
    elif name == "cfg1":
        m = M.regular_box(4, 4, 4, nxi_u=2, pressure="element", law=M.MR, materials=(2.0, 6.0))
        workload = "4x4x4 trilinear-u/element-p unit cube, MR c1=2 c2=6, FP64 Jacobian + residual"
    else:
        raise SystemExit("unknown config " + name)
    x = M.deformed_state(m, stretch=1.1, shear=0.05, noise=0.02, pressure=-2.0, seed=4)
    return m, x, workload


def algorithmic_bytes(m, es, mixed):
    """Bytes one assembly must move: Jacobian values written once (FP32 uu +
    FP64 coupling for the mixed path, all FP64 otherwise), the residual
    written once, and the coordinates / dofs / materials read once.  Index
    arrays are not counted."""
    rows = es.ndofs
    if mixed:
        jac = 4 * es.nnz_uu + 8 * es.nnz_coupling
    else:
        jac = 8 * es.nnz
    inputs = 8 * (3 * m.nu + 3 * m.nu + m.n_pressure) + 8 * m.materials.size
    return jac + 8 * rows + inputs


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.lines = []
        self.proc = None
        self.window = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))

    def wait_first_sample(self, limit_s=5.0):
        """Blocks until nvidia-smi has printed its first line (it takes a
        moment to start), so the timed region is covered by samples."""
        t0 = time.perf_counter()
        while self.proc and not self.lines and time.perf_counter() - t0 < limit_s:
            time.sleep(0.02)

    def mark(self, t0, t1):
        self.window = (t0, t1)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        lines = self.lines
        if self.window:
            inside = [ln for t, ln in lines if self.window[0] <= t <= self.window[1] + 0.1]
            lines = inside if inside else [ln for _, ln in lines[-1:]]
        else:
            lines = [ln for _, ln in lines]
        for ln in lines:
            f = [t.strip() for t in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(m, x, rp1, col1, budget_s=12.0):
    """The FP64 CPU oracle (restatement of the reference's assembly loop with
    its bisection CSR add) timed with all host threads on whole assemblies of
    the same mesh, repeated until about budget_s of CPU work."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    P = oracle.Problem(m)
    nt = os.cpu_count() or 1
    import numpy as np
    vals = np.zeros(int(rp1[-1]) - 1)
    res = np.zeros(P.ndofs)
    lib = oracle.lib()
    t0 = time.perf_counter()
    n = 0
    while True:
        rc = lib.or_assemble(P.ref, x.ctypes.data, rp1.ctypes.data, col1.ctypes.data, vals.ctypes.data,
                             res.ctypes.data, nt)
        if rc != 0:
            raise RuntimeError("oracle assembly failed")
        n += 1
        if time.perf_counter() - t0 > budget_s or n >= 20:
            break
    dt = time.perf_counter() - t0
    # one host thread (the reference's serial per-rank loop) on a sample of the mesh
    n1 = min(m.ne, 2048)
    t1 = time.perf_counter()
    if lib.or_assemble_range(P.ref, x.ctypes.data, rp1.ctypes.data, col1.ctypes.data, vals.ctypes.data,
                             res.ctypes.data, 0, n1, 1) != 0:
        raise RuntimeError("oracle assembly failed")
    d1 = time.perf_counter() - t1
    # vals / res now hold the sampled elements only: assemble the whole mesh again for the error check
    if lib.or_assemble(P.ref, x.ctypes.data, rp1.ctypes.data, col1.ctypes.data, vals.ctypes.data,
                       res.ctypes.data, nt) != 0:
        raise RuntimeError("oracle assembly failed")
    return {"value": n * m.ne / dt, "unit": UNIT, "cores": nt, "kind": "port", "cpu": host_cpu(),
            "sample": "%d full assemblies (Jacobian+residual, FP64) of the benchmark mesh, %d threads, %.1f s" % (
                n, nt, dt),
            "single_thread": {"value": n1 / d1, "unit": UNIT, "cores": 1,
                              "sample": "the first %d elements of the mesh, one thread, %.2f s" % (n1, d1)}}, vals, res


def host_cpu():
    """Model of the host CPU and its thread count, from /proc/cpuinfo."""
    model = None
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                key = line.split(":")[0].strip().lower()
                if key in ("model name", "cpu model", "hardware"):
                    model = line.split(":", 1)[1].strip()
                    break
                if key == "cpu part" and model is None:
                    model = "Arm CPU part " + line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return {"model": model or platform.processor() or platform.machine(), "threads": os.cpu_count()}


def error_vs_oracle(es, mixed, vals_gpu, vc_gpu, r_gpu, vals_or, r_or):
    """Largest difference of the GPU assembly from the FP64 oracle's assembly
    of the same state, relative to the largest magnitude of each block."""
    import numpy as np

    def rel(a, b):
        return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))
    out = {"reference": "FP64 oracle, whole assembly of the same state", "residual": rel(r_gpu, r_or)}
    if mixed:
        from cm_gb300.newton import mixed_positions
        uu_pos, cp_pos = mixed_positions(es)
        out["uu_block_fp32"] = rel(vals_gpu.astype(np.float64), vals_or[uu_pos])
        out["coupling_blocks"] = rel(vc_gpu, vals_or[cp_pos])
    else:
        out["jacobian"] = rel(vals_gpu, vals_or)
    return out


def reference_arm(args):
    """The reference's CPU assembly (the oracle port of it, with its bisection
    CSR add) on all host threads.  One step = a bounded sample of the
    workload: 4,096 consecutive elements (a different window each step),
    assembled in colour order into the full CSR arrays."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import numpy as np
    if args.config == "cfg3":
        print(json.dumps({"impl": "reference", "unavailable": "the batched configuration has no reference "
                          "counterpart (the reference assembles one equations set per call)"}))
        return
    m, x, workload = config_mesh(args.config)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    P = oracle.Problem(m)
    rp, col = P.pattern()
    vals = np.zeros(int(rp[-1]) - 1)
    res = np.zeros(P.ndofs)
    nt = os.cpu_count() or 1
    lib = oracle.lib()
    sample = min(m.ne, 4096)
    state = {"first": 0}

    def step():
        first = state["first"]
        n = min(sample, m.ne - first)
        if lib.or_assemble_range(P.ref, x.ctypes.data, rp.ctypes.data, col.ctypes.data, vals.ctypes.data,
                                 res.ctypes.data, first, n, nt) != 0:
            raise RuntimeError("oracle assembly failed")
        state["first"] = (first + n) % m.ne
        return n
    for _ in range(args.warmup):
        step()
    done = 0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        done += step()
    dt = time.perf_counter() - t0
    value = done / dt
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": workload, "elements": m.ne, "dofs": P.ndofs, "nnz": int(rp[-1]) - 1},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nt, "kind": "port",
                         "sample": "%d elements per step (consecutive windows of the benchmark mesh), Jacobian + "
                                   "residual in FP64 with the reference's bisection CSR add, element colours "
                                   "split over %d threads" % (sample, nt)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def our_arm(args):
    import numpy as np
    import torch

    from cm_gb300 import FiniteElasticityEquationsSet
    from cm_gb300.distributed import max_over_ranks
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    m, x, workload = config_mesh(args.config)
    mixed = args.config != "cfg1" and not args.fp64
    es = FiniteElasticityEquationsSet(m)
    if args.config == "cfg5":
        from cm_gb300.newton import bottom_face_pressure
        es.set_surface_pressure(bottom_face_pressure(m, 2.0))
    dev = torch.device("cuda", local)
    xd = torch.from_numpy(x).to(dev)
    r = torch.empty(es.ndofs, dtype=torch.float64, device=dev)
    if mixed:
        vu = torch.empty(es.nnz_uu, dtype=torch.float32, device=dev)
        vc = torch.empty(es.nnz_coupling, dtype=torch.float64, device=dev)
        step = lambda: es.jacobian_evaluate_mixed(xd, vu, vc, r)  # noqa: E731
    else:
        v = torch.empty(es.nnz, dtype=torch.float64, device=dev)
        step = lambda: es.jacobian_evaluate(xd, v, r)  # noqa: E731
    stream = torch.cuda.current_stream(dev)
    for _ in range(args.warmup):
        step()
    es.check_status(xd)
    torch.cuda.synchronize(dev)

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize(dev)

    # device-resident timing
    l0 = es.launch_count()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    with ClockSampler(local) as clk:
        clk.wait_first_sample()
        w0 = time.perf_counter()
        start.record(stream)
        for _ in range(args.steps):
            step()
        end.record(stream)
        end.synchronize()
        clk.mark(w0, time.perf_counter())
    launches = es.launch_count() - l0
    es.check_status(xd)
    t = start.elapsed_time(end) / 1e3
    barrier()
    t = max_over_ranks(t, dist, dev)
    step_s = t / args.steps
    value = world * m.ne / step_s

    # the same mixed assembly with double-float high-precision phases
    dfloat = None
    if mixed:
        es.set_high_precision("double_float")
        step()
        torch.cuda.synchronize(dev)
        s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s0.record(stream)
        for _ in range(args.steps):
            step()
        s1.record(stream)
        s1.synchronize()
        es.check_status(xd)
        tdf = s0.elapsed_time(s1) / 1e3 / args.steps
        dfloat = {"value": m.ne / tdf, "unit": UNIT, "ms_per_step": 1e3 * tdf,
                  "dtype": "fp32+double-float (FP32 pairs, ~48-bit) residual/coupling",
                  "roofline_frac_hbm": algorithmic_bytes(m, es, True) / tdf / 1e9 / peaks()["hbm_gbs"]}
        es.set_high_precision("fp64")

    # FP64 path on the same workload (the plain comparator)
    plain = None
    if mixed:
        v64 = torch.empty(es.nnz, dtype=torch.float64, device=dev)
        es.jacobian_evaluate(xd, v64, r)
        torch.cuda.synchronize(dev)
        k64 = max(2, args.steps // 4)
        s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s0.record(stream)
        for _ in range(k64):
            es.jacobian_evaluate(xd, v64, r)
        s1.record(stream)
        s1.synchronize()
        t64 = s0.elapsed_time(s1) / 1e3 / k64
        plain = {"value": m.ne / t64, "unit": UNIT, "ms_per_step": 1e3 * t64, "dtype": "f64",
                 "roofline_frac_hbm": algorithmic_bytes(m, es, False) / t64 / 1e9 / peaks()["hbm_gbs"]}
        del v64
        torch.cuda.empty_cache()

    # end-to-end through the C ABI with pinned host buffers
    xh = torch.from_numpy(x).pin_memory().numpy()
    rh = torch.empty(es.ndofs, dtype=torch.float64).pin_memory().numpy()
    if mixed:
        vuh = torch.empty(es.nnz_uu, dtype=torch.float32).pin_memory().numpy()
        vch = torch.empty(es.nnz_coupling, dtype=torch.float64).pin_memory().numpy()
        e2e_step = lambda: es.jacobian_evaluate_mixed(xh, vuh, vch, rh)  # noqa: E731
        d2h = 4 * es.nnz_uu + 8 * es.nnz_coupling + 8 * es.ndofs
    else:
        vh = torch.empty(es.nnz, dtype=torch.float64).pin_memory().numpy()
        e2e_step = lambda: es.jacobian_evaluate(xh, vh, rh)  # noqa: E731
        d2h = 8 * es.nnz + 8 * es.ndofs
    e2e_step()
    k_e2e = max(3, min(args.steps, 10))
    barrier()
    t0 = time.perf_counter()
    for _ in range(k_e2e):
        e2e_step()
    te = time.perf_counter() - t0
    te = max_over_ranks(te, dist, dev)
    e2e = {"value": world * m.ne * k_e2e / te, "unit": UNIT, "h2d_bytes_per_step": 8 * es.ndofs,
           "d2h_bytes_per_step": d2h, "ms_per_step": 1e3 * te / k_e2e}
    if mixed:
        # the other host-output modes of the same call, for comparison
        e2e["host_output"] = "streamed"
        others = {}
        for mode in ("in_place", "after"):
            es.set_host_output(mode)
            e2e_step()
            t0 = time.perf_counter()
            for _ in range(k_e2e):
                e2e_step()
            others[mode] = {"ms_per_step": 1e3 * (time.perf_counter() - t0) / k_e2e}
        es.set_host_output("streamed")
        e2e["other_host_outputs"] = others
        # the host link for comparison: plain device-to-host copies of the same
        # result arrays into the same pinned buffers
        srcs = [(vu, torch.from_numpy(vuh)), (vc, torch.from_numpy(vch)), (r, torch.from_numpy(rh))]
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        for _ in range(3):
            for a_, b_ in srcs:
                b_.copy_(a_, non_blocking=True)
        torch.cuda.synchronize(dev)
        tl = (time.perf_counter() - t0) / 3
        e2e["host_link"] = {"d2h_copy_ms": 1e3 * tl, "d2h_copy_gbs": d2h / tl / 1e9,
                            "note": "plain pinned device-to-host copies of the same result bytes"}

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    B = algorithmic_bytes(m, es, mixed)
    pk = peaks()
    achieved = B / step_s / 1e9
    traffic = None
    tp = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tp):
        try:
            entry = json.load(open(tp)).get(args.config + ("_mixed" if mixed else "_fp64"))
            traffic = None if entry is None else entry["bytes_per_launch"]
        except (ValueError, OSError, KeyError, TypeError):
            traffic = None
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * step_s, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32+fp64" if mixed else "f64", "data": "synthetic",
        "config": {"workload": workload, "elements": m.ne, "dofs": es.ndofs, "nnz": es.nnz,
                   "precision": "mixed: FP32 uu tangent, FP64 residual/coupling" if mixed else "FP64",
                   "parallelism": "replicas: the same mesh on every GPU, no collective on the data path"
                   if world > 1 else "single GPU",
                   "l2": "working set larger than L2 (Jacobian values %.2f GB)" % (B / 1e9)},
        "e2e": e2e,
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / pk["hbm_gbs"], "traffic": traffic, "peak_source": pk["source"],
                     "kernel": "fe_mixed_fused_kernel" if mixed else "fe_element_kernel",
                     "launches_per_step": launches / args.steps,
                     "algorithmic_bytes_per_launch": B * args.steps / max(launches, 1),
                     "traffic_unit": "DRAM bytes per launch (ncu, profiles/traffic.json)",
                     "algorithmic_bytes_per_step": B},
        "clocks": clk.summary(),
    }
    if plain:
        out["plain_fp64"] = plain
    if dfloat:
        out["mixed_double_float"] = dfloat
    if world == 1 and args.config == "cfg2" and args.extra:
        # the batched configurations as extra keys: 256 box meshes, and 32
        # variants of the full-size Guccione slab
        torch.cuda.empty_cache()
        out["batched_256_meshes"] = batch256_leg(dev, max(3, min(args.steps, 10)))
        torch.cuda.empty_cache()
        out["slab_variants_32"] = slab_variants_leg(dev, max(3, min(args.steps, 5)))
        torch.cuda.empty_cache()
    if world == 1 and not args.no_cpu:
        rp1, col1 = es.csr_pattern(base=1)
        out["cpu_baseline"], vals_or, r_or = cpu_baseline(m, x, rp1, col1)
        out["error_vs_oracle"] = error_vs_oracle(es, mixed, vuh if mixed else vh, vch if mixed else None, rh,
                                                 vals_or, r_or)
    if world == 1 and args.loadstep:
        del es, r, xd
        torch.cuda.empty_cache()
        if args.config == "cfg5":
            out["variants_batched"] = slab_variants_leg(dev, min(args.steps, 5))
            out["loadstep"] = slab_newton_leg(dev)
        else:
            out["loadstep"] = loadstep_leg(dev, n=args.loadstep_size, n_train=args.loadstep_train,
                                           n_test=args.loadstep_test, increments=args.loadstep_increments)
    if world == 1 and args.config == "cfg2" and args.extra and args.loadstep:
        # the configuration's own loading: 10 increments to stretch 1.2 / shear 0.1 on the same mesh,
        # plain FP64 against mixed + Eisenstat-Walker (about two minutes)
        torch.cuda.empty_cache()
        try:
            out["config2_loading"] = config2_loading_leg(dev, arms_wanted=["plain_fp64", "mixed_ew"])
        except Exception as e:  # the assembly line above stands on its own
            out["config2_loading"] = {"error": "%s: %s" % (type(e).__name__, e)}
    print(json.dumps(out))
    if dist:
        dist.destroy_process_group()


def slab_variants_leg(dev, steps, n=32, ex=64, ey=64, ez=16):
    """Material / pressure variants of the slab assembled together: n
    variants of one slab geometry (C log-uniform in [0.5, 2] kPa, cavity
    pressure uniform in [0.25, 2] kPa on z = 0; fe_clone shares the mesh
    arrays) in one batched call per assembly, replayed from a CUDA graph with
    the autotuned launch shape."""
    import numpy as np
    import torch

    from cm_gb300 import EquationsSetBatch, FiniteElasticityEquationsSet
    from cm_gb300 import mesh as M
    from cm_gb300.newton import bottom_face_pressure
    from cm_gb300.warmstart import sample_slab_parameters
    params = sample_slab_parameters(n, seed=51)
    t0 = time.perf_counter()
    m = M.guccione_slab(ex, ey, ez, seed=0)
    base = FiniteElasticityEquationsSet(m)
    meshes, sets, xs = [], [], []
    for i, (p, c) in enumerate(params):
        es = base.clone(np.array([float(c), 18.5, 3.58, 1.63]))
        es.set_surface_pressure(bottom_face_pressure(m, float(p)))
        meshes.append(m)
        sets.append(es)
        xs.append(torch.from_numpy(M.deformed_state(m, stretch=1.02, shear=0.01, noise=0.01, seed=i)).to(dev))
    setup_s = time.perf_counter() - t0
    batch = EquationsSetBatch(sets)
    vus, vcs, rs = batch.allocate(dev)
    cfg = batch.autotune(xs, vus, vcs, rs, repeats=2)
    batch.capture(xs, vus, vcs, rs)
    for _ in range(3):
        batch.replay(xs[0])
    batch.check(xs[0])
    stream = torch.cuda.current_stream(dev)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(dev)
    l0 = batch.launch_count()
    a.record(stream)
    for _ in range(steps):
        batch.replay(xs[0])
    b.record(stream)
    b.synchronize()
    launches = (batch.launch_count() - l0) / steps
    batch.check(xs[0])
    t = a.elapsed_time(b) / 1e3 / steps
    # the same assemblies as one library call per slab (16 colour launches
    # plus the surface launch each), into the same buffers
    for es, x, vu, vc, r in zip(sets, xs, vus, vcs, rs):
        es.jacobian_evaluate_mixed(x, vu, vc, r)
    torch.cuda.synchronize(dev)
    a.record(stream)
    for _ in range(steps):
        for es, x, vu, vc, r in zip(sets, xs, vus, vcs, rs):
            es.jacobian_evaluate_mixed(x, vu, vc, r)
    b.record(stream)
    b.synchronize()
    t_sep = a.elapsed_time(b) / 1e3 / steps
    ne = sum(m.ne for m in meshes)
    B = sum(algorithmic_bytes(m, s_, True) for m, s_ in zip(meshes, sets))
    return {"workload": "%d variants of the %dx%dx%d triquadratic Guccione slab (C log-U[0.5,2] kPa, cavity pressure "
                        "U[0.25,2] kPa), one batched call per assembly of all of them, from a CUDA graph"
                        % (n, ex, ey, ez),
            "elements": ne, "value": ne / t, "unit": UNIT, "ms_per_step": 1e3 * t, "graph_replays_per_step": 1,
            "kernel_launches_per_step": launches,
            "roofline_frac_hbm": B / t / 1e9 / peaks()["hbm_gbs"], "autotuned": cfg, "setup_s": setup_s,
            "separate_calls": {"value": ne / t_sep, "unit": UNIT, "ms_per_step": 1e3 * t_sep,
                               "calls_per_step": n}}


def slab_newton_leg(dev, ex=16, ey=16, ez=4, increments=8, n_train=48, n_test=4, modes=16, train_steps=4000):
    """Newton with the reference's pressure-increment rule on a Guccione slab
    (the slab configuration at reduced resolution: 40x40x10 mm, fibres -60..+60
    degrees through the thickness, lateral faces clamped, cavity pressure on
    z = 0), over seeded (pressure in [0.25, 2] kPa, C log-uniform in [0.5, 2]
    kPa): the plain method (FP64 Jacobian, `increments` pressure increments)
    against the mixed Jacobian started from the learned prediction (the full
    pressure at once, plain method as fallback), all to ||r||_2 <= 1e-10."""
    import numpy as np
    import torch

    from cm_gb300 import FiniteElasticityEquationsSet
    from cm_gb300 import mesh as M
    from cm_gb300 import newton as N
    from cm_gb300 import warmstart as W
    m = M.guccione_slab(ex, ey, ez, seed=0)
    es = FiniteElasticityEquationsSet(m)
    plain = W.SlabProblem(es, N.NewtonOptions(linear="mg"), device=dev)
    fast = W.SlabProblem(es, N.NewtonOptions(linear="mg", precision="mixed", forcing="ew"), device=dev)
    train = W.sample_slab_parameters(n_train, seed=41)
    test = W.sample_slab_parameters(n_test, seed=42)
    t0 = time.perf_counter()
    states, it_train = W.generate_solves(fast, train, increments)
    t_data = time.perf_counter() - t0
    ws = W.LearnedWarmStart(fast.n_pressure, modes=min(modes, n_train - 1), seed=0, device=dev,
                            featurize=W.slab_features)
    rep = ws.fit(train, states, steps=train_steps, lr=2e-3, batch=min(256, n_train))
    plain.solve_reference(test[0], increments)      # warm-up of both paths
    fast.solve_from_state(test[0], ws.predict(test[:1])[0], increments)
    rows = []
    for p in test:
        xp, rp, tp = plain.solve_reference(p, increments)
        t1 = time.perf_counter()
        guess = ws.predict(p[None])[0]
        xl, rl, _, ok = fast.solve_from_state(p, guess, increments)
        tl = time.perf_counter() - t1
        uz = (xp[2 * m.nu:3 * m.nu].cpu().numpy() - m.X[2])
        rows.append({"plain_iters": sum(r.iterations for r in rp), "plain_krylov": sum(sum(r.linear_iterations) for r in rp),
                     "plain_s": tp, "learned_iters": sum(r.iterations for r in rl),
                     "learned_krylov": sum(sum(r.linear_iterations) for r in rl), "learned_s": tl, "accepted": bool(ok),
                     "learned_first_residual": rl[0].residual_norms[0], "plain_first_residual": rp[0].residual_norms[0],
                     "converged": bool(rp[-1].converged and rl[-1].converged),
                     "final_residual": max(rp[-1].residual_norms[-1], rl[-1].residual_norms[-1]),
                     "max_diff": float((xl - xp).abs().max()), "max_uz": float(uz.max())})
    mean = lambda k: float(np.mean([r[k] for r in rows]))  # noqa: E731
    return {
        "workload": ("%dx%dx%d triquadratic Guccione slab 40x40x10 mm (%d dofs), lateral faces clamped, cavity "
                     "pressure U[0.25,2] kPa on z=0, C log-U[0.5,2] kPa; %d held-out problems"
                     % (ex, ey, ez, es.ndofs, n_test)),
        "plain_fp64": {"newton_iterations": mean("plain_iters"), "krylov_iterations": mean("plain_krylov"),
                       "solve_ms": 1e3 * mean("plain_s"), "load_step_ms": 1e3 * mean("plain_s") / increments,
                       "increments": increments, "guess": "reference (current field)"},
        "mixed_learned": {"newton_iterations": mean("learned_iters"), "krylov_iterations": mean("learned_krylov"),
                          "solve_ms": 1e3 * mean("learned_s"), "load_step_ms": 1e3 * mean("learned_s"),
                          "increments": 1, "accepted_guesses": int(sum(r["accepted"] for r in rows)),
                          "initial_residuals": [r["learned_first_residual"] for r in rows]},
        "solve_speedup": mean("plain_s") / mean("learned_s"),
        "all_converged_1e-10": all(r["converged"] and r["final_residual"] <= 1e-10 for r in rows),
        "max_solution_difference": max(r["max_diff"] for r in rows),
        "max_deflection_mm": max(r["max_uz"] for r in rows),
        "training": {"solves": n_train, "data_s": t_data, "mean_newton_iterations": float(it_train.mean()),
                     "modes": rep.modes, "train_loss": rep.train_loss, "train_s": rep.seconds},
    }


def loadstep_leg(dev, n=8, n_train=48, n_test=4, increments=8, modes=64, train_steps=2000):
    """Newton load-step comparison on an n^3 triquadratic box (clamped stretch
    + shear, Mooney-Rivlin, seeded parameters as in the learned-warm-start
    configuration): the plain method (FP64 Jacobian, reference initial guess,
    `increments` load increments) against the mixed Jacobian started from the
    learned prediction (one full-load increment, plain method as fallback).
    Both reach ||r||_2 <= 1e-10 on every held-out problem."""
    import numpy as np
    import torch

    from cm_gb300 import FiniteElasticityEquationsSet
    from cm_gb300 import mesh as M
    from cm_gb300 import newton as N
    from cm_gb300 import warmstart as W
    m = M.regular_box(n, n, n, nxi_u=3, pressure="node", law=M.MR, materials=(2.0, 6.0), perturb=0.1, seed=2)
    es = FiniteElasticityEquationsSet(m)
    plain = W.ParametricProblem(es, N.NewtonOptions(linear="mg"), device=dev)
    fast = W.ParametricProblem(es, N.NewtonOptions(linear="mg", precision="mixed", forcing="ew"), device=dev)
    train = W.sample_parameters(n_train, seed=21)
    test = W.sample_parameters(n_test, seed=22)
    t0 = time.perf_counter()
    states, it_train = W.generate_solves(fast, train, increments)
    t_data = time.perf_counter() - t0
    ws = W.LearnedWarmStart(fast.n_pressure, modes=min(modes, n_train - 1), seed=0, device=dev)
    rep = ws.fit(train, states, steps=train_steps, lr=2e-3, batch=min(256, n_train))
    plain.solve_reference(test[0], increments)      # warm-up of both paths
    fast.solve_from_state(test[0], ws.predict(test[:1])[0], increments)
    rows = []
    for p in test:
        xp, rp, tp = plain.solve_reference(p, increments)
        t1 = time.perf_counter()
        guess = ws.predict(p[None])[0]
        xl, rl, tl, ok = fast.solve_from_state(p, guess, increments)
        tl = time.perf_counter() - t1
        rows.append({"plain_krylov": sum(sum(r.linear_iterations) for r in rp),
                     "learned_krylov": sum(sum(r.linear_iterations) for r in rl),
                     "plain_iters": sum(r.iterations for r in rp), "plain_s": tp,
                     "plain_increment_ms": 1e3 * tp / len(rp), "learned_iters": sum(r.iterations for r in rl),
                     "learned_s": tl, "accepted": bool(ok), "converged": bool(rp[-1].converged and rl[-1].converged),
                     "max_diff": float((xl - xp).abs().max()),
                     "final_residual": max(rp[-1].residual_norms[-1], rl[-1].residual_norms[-1])})
    mean = lambda k: float(np.mean([r[k] for r in rows]))  # noqa: E731
    return {
        "workload": "%d^3 triquadratic-u/trilinear-p box (%d dofs), clamped stretch U[1,1.3] + shear U[0,0.2], "
                    "MR c1,c2 log-U[0.5,10]; %d held-out problems" % (n, es.ndofs, n_test),
        "plain_fp64": {"newton_iterations": mean("plain_iters"), "krylov_iterations": mean("plain_krylov"),
                       "solve_ms": 1e3 * mean("plain_s"),
                       "load_step_ms": mean("plain_increment_ms"), "increments": increments,
                       "jacobian": "FP64", "guess": "reference (current field)",
                       "krylov_tolerance": "1e-5 (reference default)"},
        "mixed_learned": {"newton_iterations": mean("learned_iters"), "krylov_iterations": mean("learned_krylov"),
                          "solve_ms": 1e3 * mean("learned_s"),
                          "load_step_ms": 1e3 * mean("learned_s"), "increments": 1,
                          "jacobian": "FP32 uu (BF16x3 tensor cores) + FP64 coupling/residual",
                          "guess": "POD-MLP prediction (BF16 tensor-core inference)",
                          "accepted_guesses": int(sum(r["accepted"] for r in rows)),
                          "krylov_tolerance": "Eisenstat-Walker forcing"},
        "solve_speedup": mean("plain_s") / mean("learned_s"),
        "all_converged_1e-10": all(r["converged"] and r["final_residual"] <= 1e-10 for r in rows),
        "max_solution_difference": max(r["max_diff"] for r in rows),
        "training": {"solves": n_train, "data_s": t_data, "mean_newton_iterations": float(it_train.mean()),
                     "modes": rep.modes, "pod_energy": rep.energy, "train_loss": rep.train_loss,
                     "train_s": rep.seconds},
        "linear_solver": "GMRES + block-triangular preconditioner (multigrid V-cycle in a CUDA graph, "
                         "scaled pressure mass)",
    }


def batch256_leg(dev, steps, n=256):
    """The batched configuration as an extra key of the default line: 256
    independent box meshes (seeded sizes, element types and materials) in one
    batched call per assembly replayed from a CUDA graph with the autotuned
    launch shape."""
    import torch

    from cm_gb300 import EquationsSetBatch, create_equations_sets
    from cm_gb300 import mesh as M
    from cm_gb300.distributed import rank_batch_meshes
    t0 = time.perf_counter()
    meshes, stretches = rank_batch_meshes(n, 0)
    sets = create_equations_sets(meshes)
    setup_s = time.perf_counter() - t0
    xs = [torch.from_numpy(M.deformed_state(m, stretch=st, shear=0.0, noise=0.02, pressure=-1.0, seed=i)).to(dev)
          for i, (m, st) in enumerate(zip(meshes, stretches))]
    batch = EquationsSetBatch(sets)
    vus, vcs, rs = batch.allocate(dev)
    cfg = batch.autotune(xs, vus, vcs, rs, repeats=1)
    batch.capture(xs, vus, vcs, rs)
    for _ in range(3):
        batch.replay(xs[0])
    batch.check(xs[0])
    stream = torch.cuda.current_stream(dev)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(dev)
    l0 = batch.launch_count()
    a.record(stream)
    for _ in range(steps):
        batch.replay(xs[0])
    b.record(stream)
    b.synchronize()
    launches = (batch.launch_count() - l0) / steps
    batch.check(xs[0])
    t = a.elapsed_time(b) / 1e3 / steps
    ne = sum(m.ne for m in meshes)
    B = sum(algorithmic_bytes(m, s_, True) for m, s_ in zip(meshes, sets))
    out = {"workload": "%d box meshes (edges U{4..24}, lengths U[0.5,2], trilinear/element-p or triquadratic/nodal-p "
                       "50/50, MR c1,c2 log-U[0.5,10]), one batched call per assembly from a CUDA graph" % n,
           "elements": ne, "value": ne / t, "unit": UNIT, "ms_per_step": 1e3 * t,
           "kernel_launches_per_step": launches, "roofline_frac_hbm": B / t / 1e9 / peaks()["hbm_gbs"],
           "algorithmic_bytes_per_step": B, "autotuned": cfg, "setup_s": setup_s}
    batch.close()
    return out


def config2_loading_leg(dev, increments=10, stretch=1.2, shear=0.1, arms_wanted=None):
    """The single-large-mesh configuration's loading: the 32^3 triquadratic
    box (859,812 dofs) clamped at x = 0 and moved to stretch 1.2 / shear 0.1
    on x = 1 in 10 load increments (the reference's fixed-incremented rule),
    Newton from the reference guess (the current field) to ||r||_2 <= 1e-10
    at every increment, three ways: the plain method (FP64 Jacobian, KSP
    relative tolerance 1e-5, the reference default), the mixed Jacobian with
    the same tolerance, and the mixed Jacobian with Eisenstat-Walker forcing.
    The linear solver is GMRES with the multigrid block preconditioner in all
    three, with 32-bit CSR indices."""
    import torch

    from cm_gb300 import FiniteElasticityEquationsSet
    from cm_gb300 import newton as N
    m, _, _ = config_mesh("cfg2")
    es = FiniteElasticityEquationsSet(m)
    bc = N.clamped_stretch_shear_conditions(m, stretch, shear)
    arms = {"plain_fp64": N.NewtonOptions(linear="mg", csr_index="int32"),
            "mixed": N.NewtonOptions(linear="mg", precision="mixed", csr_index="int32"),
            "mixed_ew": N.NewtonOptions(linear="mg", precision="mixed", forcing="ew", csr_index="int32")}
    if arms_wanted:
        arms = {k: v for k, v in arms.items() if k in arms_wanted}
    out, xs = {}, {}
    for name, opt in arms.items():
        solver = N.LoadStepSolver(es, bc, opt, device=dev)
        x0 = torch.from_numpy(N.initial_state(m)).to(dev)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()

        def progress(i, rep, name=name, t0=t0):
            print("config2 %s increment %d: %s, %d Newton, %d Krylov, assembly %.2f s, linear %.2f s "
                  "(multigrid set-up %.2f s), %.1f s so far"
                  % (name, i, "converged" if rep.converged else "not converged", rep.iterations,
                     sum(rep.linear_iterations), rep.assembly_seconds, rep.linear_seconds,
                     rep.preconditioner_seconds, time.perf_counter() - t0), file=sys.stderr, flush=True)
        x, reps = solver.solve(x0, increments, progress=progress)
        torch.cuda.synchronize(dev)
        t = time.perf_counter() - t0
        xs[name] = x
        out[name] = {"newton_iterations": int(sum(r.iterations for r in reps)),
                     "krylov_iterations": int(sum(sum(r.linear_iterations) for r in reps)),
                     "solve_ms": 1e3 * t, "load_step_ms": 1e3 * t / max(len(reps), 1),
                     "increments_done": len(reps),
                     "converged_1e-10": bool(all(r.converged for r in reps) and len(reps) == increments),
                     "final_residual": float(reps[-1].residual_norms[-1]),
                     "assembly_s": float(sum(r.assembly_seconds for r in reps)),
                     "linear_s": float(sum(r.linear_seconds for r in reps)),
                     "multigrid_setup_s": float(sum(r.preconditioner_seconds for r in reps))}
        del solver
        torch.cuda.empty_cache()
    if "plain_fp64" in xs:
        ref = xs["plain_fp64"]
        for name in ("mixed", "mixed_ew"):
            if name in xs:
                out[name]["max_solution_difference"] = float((xs[name] - ref).abs().max())
    out["workload"] = ("32^3 triquadratic-u/trilinear-p box (%d dofs), MR c1=2 c2=6, x=0 clamped, x=1 moved to "
                       "stretch %.2f + shear %.2f in %d increments" % (es.ndofs, stretch, shear, increments))
    if "plain_fp64" in out and "mixed_ew" in out:
        out["speedup_mixed_ew"] = out["plain_fp64"]["solve_ms"] / out["mixed_ew"]["solve_ms"]
    return out


def config4_study(dev, n=16, n_train=2048, n_test=256, n_timed=32, increments=10, modes=64, train_steps=4000):
    """The learned-warm-start configuration at its stated size: the 16^3
    triquadratic box (112,724 dofs), 2,048 training and 256 held-out
    parameter sets (stretch, shear, c1, c2) from the configuration's
    distributions, 64 POD modes, the 4-256-256-256-64 network.

    Training states are Newton solves to ||r||_2 <= 1e-10 with the mixed
    Jacobian and Eisenstat-Walker forcing (arm (iii)'s solver), each started
    from the previous training solution along a nearest-neighbour path in
    parameter space (two full-load solves at interpolated parameters, the
    reference increments where that fails): they are the converged solutions
    whatever the start or the Jacobian precision (arms (i) and (iii) agree
    to 2e-10).  Four arms on held-out problems, each to ||r||_2 <= 1e-10:
      (i)   plain: FP64 Jacobian, reference guess, `increments` increments,
            KSP relative tolerance 1e-5 (the reference default);
      (ii)  (i) with Eisenstat-Walker forcing;
      (iii) mixed Jacobian, Eisenstat-Walker, reference guess and increments;
      (iv)  mixed Jacobian, Eisenstat-Walker, the learned guess in one
            increment (arm (iii) as the fallback).
    Arm (iv) runs on all held-out problems; arms (i)-(iii) on the first
    `n_timed` of them (the same problems), which the ratios use."""
    import numpy as np
    import torch

    from cm_gb300 import FiniteElasticityEquationsSet
    from cm_gb300 import mesh as M
    from cm_gb300 import newton as N
    from cm_gb300 import warmstart as W
    t_all = time.perf_counter()
    m = M.regular_box(n, n, n, nxi_u=3, pressure="node", law=M.MR, materials=(2.0, 6.0), perturb=0.1, seed=2)
    es = FiniteElasticityEquationsSet(m)
    arms = {
        "i_plain": W.ParametricProblem(es, N.NewtonOptions(linear="mg"), device=dev),
        "ii_plain_ew": W.ParametricProblem(es, N.NewtonOptions(linear="mg", forcing="ew"), device=dev),
        "iii_mixed_ew": W.ParametricProblem(es, N.NewtonOptions(linear="mg", precision="mixed", forcing="ew"),
                                            device=dev),
    }
    learned = arms["iii_mixed_ew"]
    train = W.sample_parameters(n_train, seed=21)
    test = W.sample_parameters(n_test, seed=22)
    t0 = time.perf_counter()
    def progress(done, i, newton, sec):
        if sec > 10.0 or done % 64 == 0:
            print("config4: training solve %d/%d (row %d): %d Newton, %.1f s; %.1f s so far"
                  % (done, n_train, i, newton, sec, time.perf_counter() - t0), file=sys.stderr, flush=True)
    states, it_train = W.generate_solves(learned, train, increments, continuation=True, steps=2, progress=progress)
    t_data = time.perf_counter() - t0
    print("config4: %d training solves in %.1f s" % (n_train, t_data), file=sys.stderr, flush=True)
    ws = W.LearnedWarmStart(learned.n_pressure, modes=min(modes, n_train - 1), seed=0, device=dev)
    rep = ws.fit(train, states, steps=train_steps, lr=2e-3, batch=256)
    del states
    # warm-up of every path
    for a in arms.values():
        a.solve_reference(test[0], increments)
    learned.solve_from_state(test[0], ws.predict(test[:1])[0], increments)

    def summary(rows):
        k = len(rows)
        return {"problems": k,
                "newton_iterations": float(np.mean([r["newton"] for r in rows])),
                "krylov_iterations": float(np.mean([r["krylov"] for r in rows])),
                "solve_ms": 1e3 * float(np.mean([r["s"] for r in rows])),
                "load_step_ms": 1e3 * float(np.mean([r["s"] / r["incs"] for r in rows])),
                "all_converged_1e-10": bool(all(r["ok"] for r in rows))}

    def row(x, reps, t):
        return {"newton": sum(r.iterations for r in reps), "krylov": sum(sum(r.linear_iterations) for r in reps),
                "s": t, "incs": len(reps), "x": x,
                "ok": bool(reps[-1].converged and reps[-1].residual_norms[-1] <= 1e-10)}

    out = {}
    ref_x = []
    for name, a in arms.items():
        rows = []
        for p in test[:n_timed]:
            x, reps, t = a.solve_reference(p, increments)
            rows.append(row(x, reps, t))
        if name == "i_plain":
            ref_x = [r["x"] for r in rows]
        out[name] = summary(rows)
        out[name]["max_difference_to_i"] = float(max((r["x"] - xr).abs().max() for r, xr in zip(rows, ref_x)))
    rows, accepted = [], 0
    for p in test:
        t1 = time.perf_counter()
        guess = ws.predict(p[None])[0]
        x, reps, _, ok = learned.solve_from_state(p, guess, increments)
        t = time.perf_counter() - t1
        accepted += int(ok)
        rows.append(row(x, reps, t))
        rows[-1]["incs"] = 1
    out["iv_mixed_ew_learned"] = summary(rows)
    out["iv_mixed_ew_learned"]["accepted_guesses"] = accepted
    out["iv_mixed_ew_learned"]["max_difference_to_i"] = float(
        max((r["x"] - xr).abs().max() for r, xr in zip(rows[:n_timed], ref_x)))
    iv_timed = summary(rows[:n_timed])
    out["iv_on_timed_problems"] = iv_timed
    for name in ("i_plain", "ii_plain_ew", "iii_mixed_ew"):
        out["speedup_iv_vs_" + name] = out[name]["solve_ms"] / iv_timed["solve_ms"]
    out["workload"] = ("%d^3 triquadratic-u/trilinear-p box (%d dofs), clamped stretch U[1,1.3] + shear U[0,0.2], "
                       "MR c1,c2 log-U[0.5,10]; %d training, %d held-out problems (%d timed on every arm)"
                       % (n, es.ndofs, n_train, n_test, n_timed))
    out["training"] = {"solves": n_train, "data_s": t_data, "mean_newton_iterations": float(it_train.mean()),
                       "modes": rep.modes, "pod_energy": rep.energy, "pod_relative_error": rep.pod_relative_error,
                       "train_loss": rep.train_loss, "train_s": rep.seconds, "steps": train_steps,
                       "data": "Newton to 1e-10 (mixed Jacobian, Eisenstat-Walker), two-step continuation "
                               "along a nearest-neighbour path"}
    out["total_s"] = time.perf_counter() - t_all
    return out


def batch_arm(args):
    """Batched configuration: 256 independent box meshes assembled in one
    persistent launch (captured in a CUDA graph), launch shape from the
    autotuner."""
    import numpy as np
    import torch

    from cm_gb300 import EquationsSetBatch, create_equations_sets
    from cm_gb300 import mesh as M
    from cm_gb300.distributed import max_over_ranks, rank_batch_meshes
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    dev = torch.device("cuda", local)
    t0 = time.perf_counter()
    meshes, stretches = rank_batch_meshes(args.batch_meshes, rank)
    sets = create_equations_sets(meshes)
    setup_s = time.perf_counter() - t0
    xs_h = [M.deformed_state(m, stretch=s, shear=0.0, noise=0.02, pressure=-1.0, seed=i)
            for i, (m, s) in enumerate(zip(meshes, stretches))]
    xs = [torch.from_numpy(x).to(dev) for x in xs_h]
    batch = EquationsSetBatch(sets)
    vus, vcs, rs = batch.allocate(dev)
    cfg = batch.autotune(xs, vus, vcs, rs, repeats=2)
    batch.capture(xs, vus, vcs, rs)
    stream = torch.cuda.current_stream(dev)
    for _ in range(args.warmup):
        batch.replay(xs[0])
    batch.check(xs[0])
    torch.cuda.synchronize(dev)
    ne = sum(m.ne for m in meshes)
    l0 = batch.launch_count()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if dist:
        dist.barrier()
    torch.cuda.synchronize(dev)
    with ClockSampler(local) as clk:
        clk.wait_first_sample()
        w0 = time.perf_counter()
        start.record(stream)
        for _ in range(args.steps):
            batch.replay(xs[0])
        end.record(stream)
        end.synchronize()
        clk.mark(w0, time.perf_counter())
    launches = batch.launch_count() - l0
    batch.check(xs[0])
    t = start.elapsed_time(end) / 1e3
    t = max_over_ranks(t, dist, dev)
    step_s = t / args.steps
    B = sum(algorithmic_bytes(m, s, True) for m, s in zip(meshes, sets))
    # end to end: pinned host inputs in, assembled systems out, every step
    xh = [torch.from_numpy(x).pin_memory() for x in xs_h]
    vuh = [torch.empty(v.shape, dtype=v.dtype).pin_memory() for v in vus]
    vch = [torch.empty(v.shape, dtype=v.dtype).pin_memory() for v in vcs]
    rh = [torch.empty(v.shape, dtype=v.dtype).pin_memory() for v in rs]

    def e2e_step():
        for a, b in zip(xs, xh):
            a.copy_(b, non_blocking=True)
        batch.replay(xs[0])
        for lst_d, lst_h in ((vus, vuh), (vcs, vch), (rs, rh)):
            for a, b in zip(lst_d, lst_h):
                b.copy_(a, non_blocking=True)
        torch.cuda.synchronize(dev)
    e2e_step()
    k = max(3, min(args.steps, 10))
    te0 = time.perf_counter()
    for _ in range(k):
        e2e_step()
    te = max_over_ranks((time.perf_counter() - te0) / k, dist, dev)
    h2d = sum(8 * x.numel() for x in xh)
    d2h = sum(4 * v.numel() for v in vuh) + sum(8 * v.numel() for v in vch) + sum(8 * v.numel() for v in rh)
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    pk = peaks()
    achieved = B / step_s / 1e9
    out = {
        "metric": METRIC, "value": world * ne / step_s, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * step_s, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32+fp64", "data": "synthetic",
        "config": {"workload": "%d box meshes (edges U{4..24}, lengths U[0.5,2], trilinear/element-p or "
                               "triquadratic/nodal-p 50/50, MR c1,c2 log-U[0.5,10], stretch U[1,1.3]), "
                               "one persistent launch per assembly replayed from a CUDA graph" % len(meshes),
                   "elements": ne, "triquadratic_meshes": int(sum(m.nxi_u == 3 for m in meshes)),
                   "dofs": int(sum(s.ndofs for s in sets)), "nnz": int(sum(s.nnz for s in sets)),
                   "autotuned": cfg, "setup_s": setup_s,
                   "parallelism": ("independent shards: a different batch of %d meshes on each GPU, no collective "
                                   "on the data path" % len(meshes)) if world > 1 else "single GPU",
                   "l2": "working set larger than L2 (%.2f GB written per step)" % (B / 1e9)},
        "e2e": {"value": world * ne / te, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": 1e3 * te},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / pk["hbm_gbs"], "traffic": None, "peak_source": pk["source"],
                     "algorithmic_bytes_per_step": B},
        "clocks": clk.summary(),
    }
    print(json.dumps(out))
    if dist:
        dist.destroy_process_group()


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return {"hbm_gbs": float(d["hbm_gbs"]), "bf16_tflops": float(d["bf16_tflops"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "source": "fallback"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="cfg2", choices=["cfg2", "cfg4", "cfg1", "cfg3", "cfg5"])
    ap.add_argument("--batch-meshes", type=int, default=256, help="meshes in the batched configuration")
    ap.add_argument("--fp64", action="store_true", help="time the FP64 path instead of the mixed path")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--loadstep-size", type=int, default=8, help="elements per edge of the load-step box")
    ap.add_argument("--loadstep-train", type=int, default=48, help="training solves of the learned warm start")
    ap.add_argument("--loadstep-test", type=int, default=4, help="held-out problems timed")
    ap.add_argument("--loadstep-increments", type=int, default=8, help="load increments of the plain method")
    ap.add_argument("--no-loadstep", dest="loadstep", action="store_false",
                    help="skip the Newton load-step comparison (plain FP64 vs mixed + learned warm start)")
    ap.add_argument("--no-extra", dest="extra", action="store_false",
                    help="skip the extra legs of the default configuration (256 box meshes, 32 slab variants, "
                         "the 10-increment loading)")
    ap.add_argument("--config2-arms", default="",
                    help="comma-separated arms of --config2-loading (plain_fp64, mixed, mixed_ew; default all)")
    ap.add_argument("--config2-loading", action="store_true",
                    help="only solve the 32^3 box's 10-increment loading (plain FP64 vs mixed) and print it")
    ap.add_argument("--config4-study", action="store_true",
                    help="only run the learned-warm-start configuration at its stated size (2,048 training, "
                         "256 held-out solves of the 16^3 box, four arms) and print it")
    ap.add_argument("--config4-train", type=int, default=2048)
    ap.add_argument("--config4-test", type=int, default=256)
    ap.add_argument("--config4-timed", type=int, default=32)
    args = ap.parse_args()
    if args.config4_study:
        import torch
        torch.cuda.set_device(0)
        print(json.dumps({"config4_study": config4_study(torch.device("cuda", 0), n_train=args.config4_train,
                                                         n_test=args.config4_test, n_timed=args.config4_timed)}))
        return
    if args.config2_loading:
        import torch
        torch.cuda.set_device(0)
        arms = args.config2_arms.split(",") if args.config2_arms else None
        print(json.dumps({"config2_loading": config2_loading_leg(torch.device("cuda", 0), arms_wanted=arms)}))
        return
    if args.impl == "reference":
        reference_arm(args)
    elif args.config == "cfg3":
        batch_arm(args)
    else:
        our_arm(args)


if __name__ == "__main__":
    main()
