#!/usr/bin/env python3
"""Element-cycles/s of the plain FP64 explicit timestep on GB300.

Workload: the plane-strain multi-body perforation -- a 10 x 20 mm steel slug (J2, 800 MPa,
1 GPa linear hardening) at 700 m/s into a column of twelve 20 x 10 mm OFHC copper blocks
(Johnson-Cook) on a rigid floor under gravity, ~200k quads at 0.114 mm, penalty contact with
Coulomb friction 0.2, Weibull (m = 10) failure strains with fracture-energy softening
(G_f = 20 kJ/m^2) and erosion at full damage. One "step" is one central-difference timestep
of the whole scene. Inputs are synthetic (the scene is generated); the state (~60 MB) fits
in L2, so a 256 MB buffer is written between timed steps to flush it.

The timed window is fixed by the scene, not by the flags: both arms first run the scene to
step 400 (the slug strikes the blocks near step 73, so by then contact pairs, Johnson-Cook
solves, damage and erosion are all active), then --warmup steps, then time --steps steps. The
GPU arm and the reference arm therefore time the same steps of the same state.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference algorithm on the host cores: the C restatement of the
Java path (oracle/refcpu.c) with its assembly, gather and contact search split over every
host thread exactly as the reference's Parallel pool splits them.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

CELL = 0.114e-3
GAP = 0.5e-3
WINDOW_START = 400          # steps run before warm-up and timing, in both arms
L2_FLUSH_BYTES = 256 << 20
# DRAM bytes (read + write) of one element-pass launch of this workload in the window, from
# ncu's dram__bytes_read.sum + dram__bytes_write.sum, the mean over the launches of steps
# start + 6 and start + 7 (ncu cannot run inside the timed bench)
ELEMENT_TRAFFIC_BYTES = {CELL: (43_483_904 + 173_568 + 43_474_176 + 36_864) // 2}
# FP64-pipe warp instructions of one element-pass launch in the window: the mean of ncu's
# smsp__inst_executed_pipe_fp64.sum over the same two launches
ELEMENT_FP64_WARP_INST = {CELL: (3_078_533 + 3_061_133) // 2}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=400)
    p.add_argument("--warmup", type=int, default=20)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--cell", type=float, default=CELL)
    p.add_argument("--start", type=int, default=WINDOW_START,
                   help="steps run before the warm-up (the window's start)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-mixed", action="store_true")
    p.add_argument("--precision", default="fp64", choices=["fp64", "mixed"],
                   help="arithmetic of the headline leg (default: the reference's FP64)")
    p.add_argument("--mixed-cell", type=float, default=0.051e-3)
    p.add_argument("--mixed-steps", type=int, default=600)
    p.add_argument("--no-batched", action="store_true")
    p.add_argument("--batch-count", type=int, default=4096)
    p.add_argument("--no-adjoint", action="store_true")
    p.add_argument("--adjoint-count", type=int, default=64)
    p.add_argument("--no-burst", action="store_true")
    p.add_argument("--burst-count", type=int, default=1024)
    p.add_argument("--only", choices=["batched", "adjoint", "burst"],
                   help="run one form alone and print its JSON (profiling of small cases)")
    p.add_argument("--t-end", type=float, default=None,
                   help="with --only: the rods' run length instead of 80 us")
    p.add_argument("--batch-shape", default=None,
                   help="threads,stage_nodes,blocks_per_sm for the sweep instead of the "
                        "autotuner's choice (profiling a given shape)")
    return p.parse_args()


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def sum_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class Clocks:
    """nvidia-smi samples during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                smax = float(f[1])
            except ValueError:
                continue
            for n, v in zip(names, f[4:8]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def live_element_steps(elements, eroded0, eroded1, steps):
    return steps * (elements - 0.5 * (eroded0 + eroded1))


# Algorithmic bytes of the element kernel per element (reduced, FP64, finite strain, damage):
# connectivity 16 R; stress 32 + back stress 32 + plastic strain 8 + plastic work 8 +
# hourglass force 16, each read and written (2 x 96); damage strength, softening and failure
# strain 24 R. Per node: reference coordinates 16 + displacement 16 + velocity 16 R.
ELEMENT_BYTES = 16 + 2 * 96 + 24
NODE_BYTES = 48


WORKLOAD = ("plane-strain perforation: 10x20 mm steel slug at 700 m/s into 12 copper blocks "
            "20x10 mm on a rigid floor, gravity, penalty contact mu 0.2, Weibull m=10 damage, "
            "erosion")


def bench_config(args, E, N):
    """The workload of the line, the same dict in both arms."""
    return {"workload": WORKLOAD, "elements": E, "nodes": N, "cell_mm": args.cell * 1e3,
            "gap_mm": GAP * 1e3, "window": f"steps {args.start}+{args.warmup} .. "
                                            f"{args.start}+{args.warmup}+{args.steps}",
            "start_step": args.start,
            "l2": f"GPU arm: flushed between timed steps ({L2_FLUSH_BYTES >> 20} MB write)"}


def window_facts(s, info, t_start):
    """What the window's first step starts from: the same in both arms (the device path is
    bit-identical to the oracle)."""
    a = s._auditC()
    return {"t_start_us": t_start * 1e6, "contact_pairs": info["contact"].pairCount(),
            "yielded_fraction": a.yielded_fraction, "eroded": s.erodedElements(),
            "max_plastic_strain": a.max_plastic_strain}


def run_ours(args, world, rank, local):
    import torch
    torch.cuda.set_device(local)
    from neofiz_gb300 import build as nb
    nb.build()
    from neofiz_gb300 import ExplicitSolver, scenes

    inputs = scenes.perforation_inputs(cell=args.cell, gap=GAP)

    def positioned():
        """The scene run to the window: start + warm-up steps, on its own stream."""
        g, mesh, info = scenes.perforation_build(ExplicitSolver, inputs)
        if args.precision == "mixed":
            from neofiz_gb300 import _abi
            g.setPrecision(_abi.PRECISION_MIXED)
        stream = torch.cuda.Stream()
        g.setStream(stream.cuda_stream)
        g.run(args.start)
        g.synchronize()
        facts = window_facts(g, info, g.time())
        g.run(args.warmup)
        g.synchronize()
        return g, mesh, info, stream, facts

    g, mesh, info, stream, facts = positioned()
    E, N = mesh.elementCount, mesh.nodeCount
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    eroded0 = g.erodedElements()
    launches0 = g.launchCount()
    clocks = Clocks(local)
    barrier(world)
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.3)
    evs = []
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        g.run(1)
        b.record(stream)
        evs.append((a, b))
    torch.cuda.synchronize()
    g.synchronize()
    clk = clocks.stop()
    barrier(world)
    ms = sum(a.elapsed_time(b) for a, b in evs)
    launches = g.launchCount() - launches0
    eroded1 = g.erodedElements()
    ms_max = max_over_ranks(ms, world)
    work = live_element_steps(E, eroded0, eroded1, args.steps)
    value = world * work / (ms_max * 1e-3)
    status = g.statusWord()
    facts["eroded_during_timing"] = eroded1 - eroded0
    facts["contact_pairs_at_end"] = info["contact"].pairCount()
    end_state = (g.readField(1).tobytes(), g.time())
    del g

    # Roofline of the dominant kernel, over the same steps: a second handle run to the same
    # state (bit-identical), its timed steps bracketed group by group by events on its stream
    p, _, _, pstream, _ = positioned()
    p.profile(True)
    for _ in range(args.steps):
        with torch.cuda.stream(pstream):
            flush.zero_()
        p.run(1)
    groups, covered = p.profileRead()
    p.profile(False)
    same_window = (p.readField(1).tobytes(), p.time()) == end_state
    del p
    per_step = {k: v / max(covered, 1) for k, v in groups.items()}
    top = max(per_step, key=per_step.get)
    elem_ms = per_step["element"]
    live = E - 0.5 * (eroded0 + eroded1)
    elem_bytes = ELEMENT_BYTES * live + NODE_BYTES * N
    peaks, peak_kind = measured_peaks()
    achieved = elem_bytes / (elem_ms * 1e-3) / 1e9 if elem_ms > 0 else None
    fp64 = fp64_roofline(elem_ms, args.cell)

    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(args, torch)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(args)

    mixed = None
    if not args.no_mixed:
        mixed = run_mixed(args, torch)

    batched = None
    if not args.no_batched:
        batched = run_batched(args, plain_fp64=value)

    adjoint = None
    if not args.no_adjoint:
        adjoint = run_adjoint(args)

    burst = None
    if not args.no_burst:
        burst = run_burst(args)

    if rank == 0:
        line = {
            "metric": "element-cycles/s, plain FP64 explicit timestep (live elements x steps / s)",
            "value": value,
            "unit": "element-cycles/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": ms_max / args.steps,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f64" if args.precision == "fp64" else "f32 element arithmetic, f64 kinematics",
            "data": "synthetic (generated scene; no dataset)",
            "config": bench_config(args, E, N),
            "parallelism": f"replicas x{world}" if world > 1 else "single scene",
            "window_state": facts,
            "roofline": {
                "bound": "hbm", "kernel": "k_element_reduced_listed",
                "achieved": achieved, "peak": peaks.get("hbm_gbs"), "unit": "GB/s",
                "frac": (achieved / peaks["hbm_gbs"]) if achieved else None,
                "peak_source": peak_kind,
                "bytes_per_launch": elem_bytes, "launch_ms": elem_ms,
                "launch_ms_source": "CUDA events around the element group, same window, "
                                    "second handle (same state: " + str(same_window) + ")",
                "traffic": ELEMENT_TRAFFIC_BYTES.get(args.cell),
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum, one launch",
                "note": "FP64 arithmetic, not HBM, bounds this kernel on GB300: see fp64",
                "fp64": fp64,
                "group_ms_per_step": per_step, "top_group": top,
            },
            "cpu_baseline": cpu,
            "e2e": e2e,
            "mixed": mixed,
            "batched": batched,
            "adjoint": adjoint,
            "burst": burst,
            "clocks": clk,
            "gpu_launches": launches,
            "status_word": status,
        }
        line["summary"] = summary_of(line)
        print(json.dumps(line))


def fp64_roofline(elem_ms, cell):
    """The element pass against the device's measured FP64 pipe rate: its FP64 warp
    instructions per launch (ncu, the same window) over its event-timed duration."""
    from neofiz_gb300 import _native
    rate, flops = _native.fp64_rate()
    out = {"bound": "fp64", "unit": "FP64 warp instructions/s", "peak": rate,
           "peak_tflops": flops / 1e12,
           "peak_source": "measured in this run: nf_device_fp64_rate (DFMA chains, every SM)"}
    count = ELEMENT_FP64_WARP_INST.get(cell)
    if count and elem_ms > 0:
        achieved = count / (elem_ms * 1e-3)
        out.update({"achieved": achieved, "frac": achieved / rate,
                    "fp64_warp_inst_per_launch": count,
                    "count_source": "ncu smsp__inst_executed_pipe_fp64.sum, one launch of the "
                                    "window"})
    return out


def summary_of(line):
    """The headline figures of every leg, compact, as the line's last key."""
    def g(d, *ks):
        for k in ks:
            if not isinstance(d, dict):
                return None
            d = d.get(k)
        return d
    r = line["roofline"]
    out = {"value": line["value"], "e2e": g(line, "e2e", "value"),
           "cpu": g(line, "cpu_baseline", "value"),
           "hbm_frac": r.get("frac"), "fp64_frac": g(r, "fp64", "frac"),
           "element_ms": r.get("launch_ms")}
    if line.get("mixed"):
        m = line["mixed"]
        out["mixed"] = {"value": m["value"], "x_fp64": m["speedup_vs_fp64"],
                        "slug_v_err": g(m, "errors_vs_fp64", "slug_residual_velocity_rel"),
                        "eroded": g(m, "errors_vs_fp64", "eroded_count")}
    if line.get("batched"):
        b = line["batched"]
        out["batched"] = {"value": b["value"], "x_plain": b.get("speedup_vs_plain_fp64_path"),
                          "L_err_max": g(b, "L_over_L0_error_vs_fp64", "max"),
                          "mixed": g(b, "mixed", "value"),
                          "mixed_x_plain": g(b, "mixed", "speedup_vs_plain_fp64_path")}
    if line.get("adjoint"):
        a = line["adjoint"]
        out["adjoint"] = {"cost_one": g(a, "cost_vs_forward", "one_objective"),
                          "cost_both": g(a, "cost_vs_forward", "both_objectives"),
                          "max_rel_error": g(a, "rod0", "max_rel_error"),
                          "tube_cost": g(a, "tube", "cost_vs_forward"),
                          "tube_max_rel_error": g(a, "tube", "max_rel_error")}
    if line.get("burst"):
        b = line["burst"]
        out["burst"] = {"fp64": g(b, "fp64", "value"), "compensated": g(b, "compensated", "value")}
    return out


def run_e2e(args, torch):
    """The same metric through the public API from host buffers, for the whole job up to the
    window's end: the scene's host inputs (mesh, materials, velocities, failure strains) are
    generated first; the timed region then creates the solver from them (every upload), sets
    it up, runs start + warm-up + timed steps, and reads the nodal displacement and velocity
    fields back every 50 steps (a sampled frame) and at the end."""
    from neofiz_gb300 import ExplicitSolver, scenes
    steps = args.start + args.warmup + args.steps
    inputs = scenes.perforation_inputs(cell=args.cell, gap=GAP)
    mesh = inputs["mesh"]
    E, N = mesh.elementCount, mesh.nodeCount
    h2d = (mesh.r.nbytes + mesh.z.nbytes + mesh.conn.nbytes + 4 * E
           + inputs["vr"].nbytes + inputs["vz"].nbytes
           + inputs["failure_strain"].nbytes + inputs["fracture_energy"].nbytes)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    g, _, _ = scenes.perforation_build(ExplicitSolver, inputs)
    d2h = 0
    frames = 0
    for k in range(0, steps, 50):
        g.run(min(50, steps - k))
        for f in (g.radialDisplacement(), g.axialDisplacement(), g.velocityR(), g.velocityZ()):
            d2h += f.nbytes
        frames += 1
    g.synchronize()
    elapsed = time.perf_counter() - t0
    eroded = g.erodedElements()
    work = live_element_steps(E, 0, eroded, steps)
    return {"value": work / elapsed, "unit": "element-cycles/s",
            "h2d_bytes_per_step": h2d / steps, "d2h_bytes_per_step": d2h / steps,
            "seconds": elapsed, "frames": frames, "steps": steps,
            "note": "create + uploads + set-up + steps 0 .. window end + frame read-backs, "
                    "host wall clock"}


def _slug_velocity(g, mesh, slug):
    import numpy as np
    from neofiz_gb300 import _abi
    vr = g.velocityR()
    m = g.readField(_abi.FIELD_MASS)
    nodes = np.unique(mesh.conn.reshape(-1, 4)[slug].reshape(-1))
    return float(np.sum(m[nodes] * vr[nodes]) / np.sum(m[nodes]))


def _balance(g, info, k0):
    a = g._auditC()
    w, c = info["wall"], info["contact"]
    return (a.centred_kinetic_energy + a.strain_energy + a.plastic_dissipation
            + a.hourglass_energy + g.erodedEnergy() + w.energyLoss() + w.frictionDissipation()
            + c.dissipation() + c.energy()) / k0


def run_mixed(args, torch):
    """The mixed-precision form on the 1M-quad perforation (FP32 element arithmetic and
    state, FP64 kinematics and audits): element-cycles/s over the last steps of a run from
    t = 0, and its errors against the FP64 path run from the same inputs for the same steps."""
    from neofiz_gb300 import ExplicitSolver, _abi, scenes
    inputs = scenes.perforation_inputs(cell=args.mixed_cell, gap=GAP)
    mesh = inputs["mesh"]
    E = mesh.elementCount
    steps = args.mixed_steps
    timed = max(50, steps // 4)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    out = {}
    for prec in (_abi.PRECISION_FP64, _abi.PRECISION_MIXED):
        g, _, info = scenes.perforation_build(ExplicitSolver, inputs)
        stream = torch.cuda.Stream()
        g.setStream(stream.cuda_stream)
        g.setPrecision(prec)
        k0 = g.kineticEnergy()
        g.run(steps - timed)
        g.synchronize()
        e0 = g.erodedElements()
        ms = 0.0
        for _ in range(timed):
            with torch.cuda.stream(stream):
                flush.zero_()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            g.run(1)
            b.record(stream)
            stream.synchronize()
            ms += a.elapsed_time(b)
        e1 = g.erodedElements()
        out[prec] = {"rate": live_element_steps(E, e0, e1, timed) / (ms * 1e-3),
                     "ms_per_step": ms / timed, "slug_velocity": _slug_velocity(g, mesh, info["slug"]),
                     "eroded": e1, "balance": _balance(g, info, k0),
                     "status": g.statusWord()}
        del g
    f64, mp = out[_abi.PRECISION_FP64], out[_abi.PRECISION_MIXED]
    return {
        "workload": f"the perforation at {args.mixed_cell * 1e3:.3f} mm cells, {E} quads, "
                    f"{steps} steps from t=0 (last {timed} timed, L2 flushed)",
        "value": mp["rate"], "unit": "element-cycles/s", "ms_per_step": mp["ms_per_step"],
        "fp64_same_scene": f64["rate"], "fp64_ms_per_step": f64["ms_per_step"],
        "speedup_vs_fp64": mp["rate"] / f64["rate"],
        "errors_vs_fp64": {
            "slug_residual_velocity_rel": abs(mp["slug_velocity"] - f64["slug_velocity"])
                                          / abs(f64["slug_velocity"]),
            "eroded_count": [mp["eroded"], f64["eroded"]],
            "energy_balance": [mp["balance"], f64["balance"]],
        },
        "status_words": [f64["status"], mp["status"]],
    }


def run_batched(args, plain_fp64=None):
    """The batched Taylor sweep: args.batch_count axisymmetric rods (nr 6..24, nz 30..120,
    Johnson-Cook A, B, n, C within +-20 %, friction 0..0.2, 150..250 m/s, drawn by SplitMix64
    from a fixed seed), each run to 80 us, in one handle: autotuned shape, graph-replayed
    chunks of the persistent kernel. Its state (~0.7 GB) is larger than L2. Two reduced-
    precision forms: mixed (FP32 element arithmetic, FP64 nodal update and gather) and
    compensated (also the nodal update and gather in FP32, displacements as compensated float
    pairs); the line's value is the compensated form. Errors in L/L0 against FP64 on every
    eighth rod (the FP64 batch, whose instances are bit-identical to single-scene FP64 runs;
    checked here on four rods); the FP64 baselines are that batch and a loop of plain
    single-scene FP64 runs on a sample of eight rods."""
    import numpy as np
    from neofiz_gb300 import ExplicitSolver, _abi, scenes
    from neofiz_gb300.batch import BatchSolver
    rods = scenes.taylor_sweep(args.batch_count)
    if args.t_end:
        for r in rods:
            r["t_end"] = args.t_end
    L0 = 25.0e-3
    # one process per GPU: each rank steps its share of the rods (no collective in the data
    # path); element-steps are summed and the time is the slowest rank's
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        from neofiz_gb300.shard import shard
        mine = shard(scenes.sweep_instances(rods), world, rank, 0.6)
        rods = [rods[i] for i in mine]

    def make(sel, prec):
        return BatchSolver(scenes.sweep_instances(sel), scenes.Formulation.AXISYMMETRIC,
                           cfl=0.6, precision=prec)

    def timed(prec):
        b = make(rods, prec)
        t0 = time.perf_counter()
        shape = None
        if args.batch_shape:
            t, sn, bps = (int(x) for x in args.batch_shape.split(","))
            try:
                b.setConfig(t, sn, bps, b.config()["chunk_steps"])
                shape = b.config()
            except ValueError:          # not a valid shape for this form: tune instead
                shape = None
        if shape is None:
            shape = b.tune(64)
        tune_s = time.perf_counter() - t0
        clocks = Clocks(0)
        clocks.start()
        launches0 = b.launchCount()
        barrier(world)
        ms = max_over_ranks(b.run(), world)
        clk = clocks.stop()
        out = {"ms": ms, "cycles": int(sum_over_ranks(float(b.elementCycles()), world)),
               "state": b.state(),
               "L": np.array([m.length for m in b.measure()]) / L0,
               "launches": b.launchCount() - launches0, "shape": shape, "tune_s": tune_s,
               "clocks": clk}
        b.close()
        return out

    runs = {"compensated": timed(_abi.PRECISION_COMPENSATED), "mixed": timed(_abi.PRECISION_MIXED)}

    sub = list(range(0, len(rods), 8))
    f = make([rods[k] for k in sub], _abi.PRECISION_FP64)
    ms64 = f.run()
    cycles64 = f.elementCycles()
    L64 = np.array([m.length for m in f.measure()]) / L0
    ur64 = [f.readInstance(_abi.FIELD_UZ, j) for j in range(4)]
    f.close()
    identical = True
    loop_cycles, loop_s = 0, 0.0
    for j, k in enumerate(sub[:4]):
        s, mesh, _ = scenes.sweep_rod(ExplicitSolver, rods[k])
        s.runUntil(rods[k]["t_end"])
        identical &= bool(np.array_equal(s.readField(_abi.FIELD_UZ), ur64[j]))
    for k in range(0, len(rods), max(1, len(rods) // 8)):
        s, mesh, _ = scenes.sweep_rod(ExplicitSolver, rods[k])
        s.runUntil(1.0e-9)
        s.synchronize()
        t0 = time.perf_counter()
        s.runUntil(rods[k]["t_end"])
        s.synchronize()
        loop_s += time.perf_counter() - t0
        loop_cycles += mesh.elementCount * (s.steps() - 1)
    loop_rate = loop_cycles / loop_s
    batch64 = cycles64 / (ms64 * 1e-3)

    def summary(r):
        rate = r["cycles"] / (r["ms"] * 1e-3)
        err = np.abs(r["L"][sub] - L64) / L64
        st = r["state"]
        o = {"value": rate, "unit": "element-cycles/s", "ms": r["ms"],
             "element_cycles": r["cycles"],
             "steps_per_rod": {"mean": float(st["steps"].mean()), "max": int(st["steps"].max())},
             "shape": r["shape"], "tune_s": r["tune_s"], "gpu_launches": r["launches"],
             "speedup_vs_fp64_loop": rate / loop_rate,
             "speedup_vs_fp64_batched": rate / batch64,
             "L_over_L0_error_vs_fp64": {"max": float(err.max()), "median": float(np.median(err)),
                                         "p99": float(np.percentile(err, 99)), "rods": len(sub)},
             "status": int(st["status"].max()), "clocks": r["clocks"]}
        if plain_fp64:
            o["speedup_vs_plain_fp64_path"] = rate / plain_fp64
        return o

    comp = summary(runs["compensated"])
    if world > 1:
        comp["ranks"] = world
        comp["sharding"] = "by instance, cost-balanced (neofiz_gb300.shard); errors on rank 0's share"
    line = {
        "workload": f"{len(rods)} axisymmetric Taylor rods (nr 6..24, nz 30..120, JC +-20 %, "
                    f"mu 0..0.2, 150..250 m/s, SplitMix64 seed {scenes.SWEEP_SEED}) to 80 us, "
                    f"one handle",
        "precision": "compensated (FP32 element, nodal and gather arithmetic; displacements "
                     "as compensated float pairs; FP64 time, step and audits)",
        **comp,
        "elements": int(sum(r["nr"] * r["nz"] for r in rods)),
        "l2": "state ~0.7 GB, larger than L2; no flush",
        "mixed": summary(runs["mixed"]),
        "fp64_batched": {"value": batch64, "rods": len(sub)},
        "fp64_loop": {"value": loop_rate, "rods": len(range(0, len(rods), max(1, len(rods) // 8))),
                      "note": "plain single-scene FP64 runs one after another (runUntil), "
                              "host wall clock"},
        "fp64_batch_equals_single_scene": identical,
    }
    return line


def run_adjoint(args):
    """The adjoint gradient batch: args.adjoint_count rods with the 10 x 60 rod's mesh, 200 m/s
    and 80 us, Johnson-Cook constants and friction drawn as in the sweep. Times the plain FP64
    batched forward run, the adjoint's checkpointed forward pass (every 200 steps) and one
    backward pass per objective (L/L0, mushroom diameter); checks rod 0's gradients against
    central differences (h = 1e-6 and 1e-5 relative) of FP64 runs of exactly the forward's
    step count, perturbed one parameter at a time (batched)."""
    import dataclasses
    import numpy as np
    from neofiz_gb300 import _abi, scenes
    from neofiz_gb300.batch import BatchSolver
    rods = scenes.adjoint_rods(args.adjoint_count)
    if args.t_end:
        for r in rods:
            r["t_end"] = args.t_end

    def make(insts):
        return BatchSolver(insts, scenes.Formulation.AXISYMMETRIC, cfl=0.6)

    p = make(scenes.sweep_instances(rods))
    plain_ms = p.run()
    steps = p.state()["steps"]
    p.close()
    a = make(scenes.sweep_instances(rods))
    fwd_ms = a.adjointForward(200)
    grads, values, back_ms = {}, {}, {}
    for obj, name in ((_abi.OBJECTIVE_LENGTH_RATIO, "length_ratio"),
                      (_abi.OBJECTIVE_MUSHROOM, "mushroom_diameter")):
        v, g = a.adjointBackward(obj)
        values[name], grads[name] = v, g
        back_ms[name] = a.adjointElapsed()[1]
    # both objectives through one recompute (each bit-identical to its own pass)
    vb, gb = a.adjointBackwardMany([_abi.OBJECTIVE_LENGTH_RATIO, _abi.OBJECTIVE_MUSHROOM])
    back_ms["both_in_one_pass"] = a.adjointElapsed()[1]
    same = bool(np.array_equal(gb[0], grads["length_ratio"])
                and np.array_equal(gb[1], grads["mushroom_diameter"]))
    a.close()
    # central differences on rod 0, the perturbed runs batched
    N = int(steps[0])
    jc0 = scenes._rod_jc(rods[0])
    mat0 = scenes.rod_material_with(jc0)
    p0 = {"A": jc0.a, "B": jc0.b, "n": jc0.n, "C": jc0.c, "m": jc0.m,
          "kinematic": mat0.kinematicHardening, "friction": rods[0]["mu"]}
    names = _abi.PARAM_NAMES[:7]                    # the rods have no damage
    fd = {}
    for h in (1e-6, 1e-5):
        insts = []
        for name in names:
            for sgn in (1.0, -1.0):
                inst = scenes.sweep_instances(rods[:1])[0]
                val = p0[name] * (1.0 + sgn * h)
                if name in ("A", "B", "n", "C", "m"):
                    f = {"A": "a", "B": "b", "n": "n", "C": "c", "m": "m"}[name]
                    inst.material = scenes.rod_material_with(
                        dataclasses.replace(jc0, **{f: val})).withKinematicHardening(
                            mat0.kinematicHardening)
                elif name == "kinematic":
                    inst.material = mat0.withKinematicHardening(val)
                else:
                    inst.wall = (0.0, val)
                inst.t_end = 1.0
                insts.append(inst)
        b = make(insts)
        b.run(max_steps=N)
        m = b.measure()
        b.close()
        fd[h] = np.array([[(m[2 * k].length - m[2 * k + 1].length) / 25.0e-3,
                           m[2 * k].mushroom_diameter - m[2 * k + 1].mushroom_diameter]
                          for k in range(len(names))])
        fd[h] /= np.array([[2.0 * p0[nm] * h] * 2 for nm in names])
    ad = np.stack([grads["length_ratio"][0][:7], grads["mushroom_diameter"][0][:7]], axis=1)
    err = np.abs(ad - fd[1e-6]) / np.abs(fd[1e-6])
    scatter = np.abs(fd[1e-5] - fd[1e-6]) / np.abs(fd[1e-6])
    per = {nm: {"adjoint_vs_fd_rel": [float(err[k, 0]), float(err[k, 1])],
                "fd_scatter_h1e-5_vs_1e-6": [float(scatter[k, 0]), float(scatter[k, 1])]}
           for k, nm in enumerate(names)}
    both = fwd_ms + back_ms["both_in_one_pass"]
    tube = run_tube_adjoint(args)
    return {
        "tube": tube,
        "workload": f"{len(rods)} Taylor rods, 10x60 quads, 200 m/s, 80 us (mean "
                    f"{float(steps.mean()):.0f} steps), JC and friction drawn (seed "
                    f"{scenes.ADJOINT_SEED}); FP64; checkpoints every 200 steps",
        "parameters": list(_abi.PARAM_NAMES),
        "forward_ms": plain_ms, "adjoint_forward_ms": fwd_ms, "backward_ms": back_ms,
        "cost_vs_forward": {"one_objective": (fwd_ms + back_ms["length_ratio"]) / plain_ms,
                            "both_objectives": both / plain_ms,
                            "both_as_two_passes": (fwd_ms + back_ms["length_ratio"]
                                                   + back_ms["mushroom_diameter"]) / plain_ms},
        "one_pass_equals_two": same,
        "rod0": {"values": {k: float(v[0]) for k, v in values.items()},
                 "gradients": {k: [float(x) for x in g[0]] for k, g in grads.items()},
                 "gradients_fraction_convention": {
                     k: [float(x) for x in scenes.fraction_gradients(g[0], rods[0])]
                     for k, g in grads.items()},
                 "central_differences": per,
                 "max_rel_error": float(err.max())},
    }


def run_burst(args):
    """A burst sweep (BurstCase.run over a BarlowSweep-like grid): args.burst_count
    two-element wall slices, slenderness 15..60 and mean radius 10..40 mm drawn by SplitMix64,
    OFHC copper, ramp to 1.06 x the closed-form burst pressure, each run on the device until
    its capacity has turned over (BurstCase's sampling every 250 steps). FP64 (bit-identical to
    the reference's per-case runs) and compensated; the CPU leg is the oracle on four tubes."""
    import numpy as np
    from neofiz_gb300 import _abi, scenes
    from neofiz_gb300.batch import BatchSolver
    from oracle.oracle import OracleBatch
    rng = scenes.SplitMix64(20250703)
    pars = [(rng.uniform(15.0, 60.0), rng.uniform(10.0e-3, 40.0e-3))
            for _ in range(args.burst_count)]
    tubes = [scenes.burst_instance(mean_radius=r, slenderness=sl) for sl, r in pars]
    radius = np.array([r for _, r in pars])
    out = {}
    for name, prec in (("fp64", _abi.PRECISION_FP64),
                       ("compensated", _abi.PRECISION_COMPENSATED)):
        b = BatchSolver(tubes, scenes.Formulation.AXISYMMETRIC, cfl=scenes.BURST_CFL,
                        precision=prec)
        b.setBurst(scenes.BURST_SAMPLE_STEPS, radius, scenes.BURST_PEAK_MARGIN)
        shape = b.tune(64)
        b.setBurst(scenes.BURST_SAMPLE_STEPS, radius, scenes.BURST_PEAK_MARGIN)
        ms = b.run()
        res = b.burstResults()
        cycles = b.elementCycles()
        exact = np.array([t.pressure[0] for t in tubes]) / scenes.BURST_OVERSHOOT
        dev = 100.0 * (res["peak_capacity"] / exact - 1.0)
        out[name] = {"value": cycles / (ms * 1e-3), "unit": "element-cycles/s", "ms": ms,
                     "element_cycles": cycles, "shape": shape,
                     "traversed": int(res["traversed"].sum()), "tubes": len(tubes),
                     "steps_mean": float(b.state()["steps"].mean()),
                     "peak_vs_closed_form_pct": {"median": float(np.median(dev)),
                                                 "min": float(dev.min()), "max": float(dev.max())},
                     "peaks": res["peak_capacity"]}
        b.close()
    rel = np.abs(out["compensated"].pop("peaks") / out["fp64"]["peaks"] - 1.0)
    out["fp64"].pop("peaks")
    out["compensated"]["peak_capacity_vs_fp64"] = {"max": float(rel.max()),
                                                   "median": float(np.median(rel))}
    o = OracleBatch(tubes[:4], scenes.Formulation.AXISYMMETRIC, cfl=scenes.BURST_CFL)
    o.setBurst(scenes.BURST_SAMPLE_STEPS, radius[:4], scenes.BURST_PEAK_MARGIN)
    o.run()
    ocyc = o.elementCycles()
    out["cpu_oracle"] = {"value": ocyc / (o.elapsed() * 1e-3), "unit": "element-cycles/s",
                         "tubes": 4, "kind": "port", "threads": "one per tube"}
    out["workload"] = (f"{len(tubes)} burst slices (8 x 2 quads), slenderness 15..60, mean radius "
                       "10..40 mm, OFHC copper, ramp to 1.06 x burst over 20 ring periods, "
                       "sampled every 250 steps until the capacity turns over")
    return out


def run_tube_adjoint(args):
    """The tube of the gradient batch: QuadMesh.cylinderWall(19.6, 20.4, 40 mm, 4, 200) in
    OFHC copper (quasi-static Johnson-Cook law), smoothstep ramp to 60 MPa over 20 us,
    relaxation damping, Weibull failure strains (seed 7, scale 0.08, so damage begins before
    the capacity peak) and G_f = 60 kJ/m^2; the wall capacity (BurstCase.loadCapacity) sampled
    every 10 steps to 60 us. The gradient of its peak with respect to A, B, n and G_f,
    against central differences (h = 1e-6)."""
    import dataclasses
    import numpy as np
    from neofiz_gb300 import _abi, scenes
    from neofiz_gb300.batch import BatchSolver
    from neofiz_gb300.materials import JohnsonCook
    t_end = args.t_end if args.t_end else 60.0e-6
    law0 = JohnsonCook.COPPER_OFHC.quasiStatic()

    def tube(name=None, value=None):
        law, gf = law0, scenes.TUBE_GF
        if name in ("A", "B", "n"):
            law = dataclasses.replace(law0, **{{"A": "a", "B": "b", "n": "n"}[name]: value})
        elif name == "fracture_energy":
            gf = value
        return scenes.tube_instance(nz=200, height=40.0e-3, t_end=t_end, scale=0.08,
                                    material=scenes.tube_material(law), gf=gf)

    def make(insts):
        return BatchSolver(insts, scenes.Formulation.AXISYMMETRIC, cfl=0.5)

    p = make([tube()])
    plain_ms = p.run()
    steps = int(p.state()["steps"][0])
    p.close()
    a = make([tube()])
    fwd_ms = a.adjointForward(200, 10)
    v, g = a.adjointBackward(_abi.OBJECTIVE_PEAK_CAPACITY)
    back_ms = a.adjointElapsed()[1]
    a.close()
    p0 = {"A": law0.a, "B": law0.b, "n": law0.n, "fracture_energy": scenes.TUBE_GF}
    h = 1.0e-6
    insts = [tube(nm, p0[nm] * (1.0 + s * h)) for nm in p0 for s in (1.0, -1.0)]
    f = make(insts)
    f.adjointForward(200, 10)
    fv, _ = f.adjointBackward(_abi.OBJECTIVE_PEAK_CAPACITY)
    f.close()
    out = {}
    for k, nm in enumerate(p0):
        fd = (fv[2 * k] - fv[2 * k + 1]) / (2.0 * p0[nm] * h)
        ad = g[0][_abi.PARAM_NAMES.index(nm)]
        out[nm] = {"adjoint": float(ad), "fd": float(fd), "rel": float(abs(ad - fd) / abs(fd))}
    return {"workload": "tube 4x200 quads (40 mm), copper, 60 MPa smoothstep ramp over 20 us, "
                        f"damping, Weibull damage (scale 0.08), {steps} steps, capacity sampled "
                        "every 10 steps",
            "peak_capacity_pa": float(v[0]), "forward_ms": plain_ms,
            "adjoint_forward_ms": fwd_ms, "backward_ms": back_ms,
            "cost_vs_forward": (fwd_ms + back_ms) / plain_ms,
            "gradients_vs_central_differences": out,
            "max_rel_error": max(o["rel"] for o in out.values())}


def oracle_scene(args):
    """The oracle's copy of the scene on every host core."""
    from neofiz_gb300 import scenes
    from oracle.oracle import OracleSolver
    cores = os.cpu_count() or 1
    s, mesh, info = scenes.perforation(OracleSolver, cell=args.cell, gap=GAP)
    s.setThreads(cores)
    return s, mesh, info, cores


def cpu_baseline(args, budget_s=12.0):
    """The reference algorithm on this host's cores (oracle, threaded as the reference's
    Parallel pool), on the same scene from the window's start; a bounded sample of steps."""
    s, mesh, _, cores = oracle_scene(args)
    s.run(args.start)
    done, t = 0, 0.0
    eroded0 = s.erodedElements()
    while t < budget_s and done < 2000:
        t0 = time.perf_counter()
        s.run(5)
        t += time.perf_counter() - t0
        done += 5
    work = live_element_steps(mesh.elementCount, eroded0, s.erodedElements(), done)
    return {"value": work / t, "unit": "element-cycles/s", "cores": cores, "kind": "port",
            "sample": f"steps {args.start} .. {args.start + done} of the "
                      f"{mesh.elementCount}-quad perforation, {t:.1f} s, {cores} threads"}


def run_reference(args, world, rank):
    """The reference arm: the oracle (the C restatement of the Java path, threaded as its
    Parallel pool) on every host core, timing exactly the GPU arm's window. Its e2e is the
    whole job to the window's end (set-up and every step), as the GPU arm's e2e is."""
    if rank != 0:
        return
    t_all = time.perf_counter()
    s, mesh, info, cores = oracle_scene(args)
    E, N = mesh.elementCount, mesh.nodeCount
    s.run(args.start)
    facts = window_facts(s, info, s.time())
    s.run(args.warmup)
    eroded0 = s.erodedElements()
    t0 = time.perf_counter()
    s.run(args.steps)
    t1 = time.perf_counter()
    eroded1 = s.erodedElements()
    facts["eroded_during_timing"] = eroded1 - eroded0
    facts["contact_pairs_at_end"] = info["contact"].pairCount()
    value = live_element_steps(E, eroded0, eroded1, args.steps) / (t1 - t0)
    all_steps = args.start + args.warmup + args.steps
    e2e = live_element_steps(E, 0, eroded1, all_steps) / (t1 - t_all)
    sample = (f"steps {args.start + args.warmup} .. {all_steps} of the {E}-quad perforation, "
              f"{t1 - t0:.2f} s, {cores} threads")
    line = {
        "impl": "reference",
        "metric": "element-cycles/s, plain FP64 explicit timestep (live elements x steps / s)",
        "value": value, "unit": "element-cycles/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": (t1 - t0) * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (generated scene; no dataset)",
        "config": bench_config(args, E, N),
        "window_state": facts,
        "cpu_baseline": {"value": value, "unit": "element-cycles/s", "cores": cores,
                         "kind": "port", "sample": sample},
        "e2e": {"value": e2e, "unit": "element-cycles/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0, "seconds": t1 - t_all, "steps": all_steps,
                "note": "set-up + steps 0 .. window end, host wall clock"},
    }
    print(json.dumps(line))


def main():
    args = parse()
    world, rank, local = dist_setup()
    if args.only:
        from neofiz_gb300 import build as nb
        nb.build()
        out = {"batched": run_batched, "adjoint": run_adjoint, "burst": run_burst}[args.only](args)
        print(json.dumps(out))
        return
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
