"""Benchmark of the exaDEM per-timestep hot path on one GB300 (particle-steps/s).

Workload: 2,000,000 polydisperse spheres (radii U[0.4, 0.6]) periodic in x/y
with a floor wall, Hooke + linear cohesion + rolling kr, dt = 5e-4, seeded
random sequential addition (exadem_gb300.workloads.spheres_floor).  A step is
one Verlet iteration of the reference deck: prolog, displacement trigger and
(when triggered) neighbour rebuild, reset, gravity, contact law, gather,
force_to_accel, epilog.

Pre-roll: before any timing, each workload runs a fixed number of untimed
steps (``--preroll``, independent of ``--warmup``).  For the spheres it is 3000
steps (1.5 s of deposition): the RSA column (solid fraction 0.30, the random
sequential addition jams near 0.38) has collapsed into a bed at a solid
fraction of about 0.6 over its height, the contact count has reached its
plateau and the bed still moves enough to trigger a neighbour rebuild every
ten steps or so.  The timed window starts there.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--preroll P] [--impl native|reference] [--n N]

Prints one JSON line.  `value` is device-resident throughput (inputs already in
HBM, CUDA events on the library's stream); `e2e` is the same metric through
the public C ABI from pinned host buffers holding the pre-rolled state, with
the host->device upload, the first force pass and the device->host readback
inside the timed region.  `vs_plain` times the plain FP64 operator kernels on
the same pre-rolled state and checks that both paths end in the same bits.
`--impl reference` times the CPU restatement of the reference algorithm
(OpenMP, all host cores) on a periodic patch of the same workload, pre-rolled
the same way.  With N > 1 (torchrun) every rank runs an independent replica:
the path does not shard.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s on 1 GB300, learned+batched vs plain GPU path, same accuracy"
UNIT = "particle-steps/s"
# Algorithmic bytes of the contact kernel per interaction: history friction +
# moment read and written (2 x 48 B) + two u32 particle indices.
CONTACT_BYTES_PER_INTERACTION = 104
# Algorithmic bytes of the particle integration per particle-step (prolog and
# epilog together): read r, v, omega, alpha, q, a (19 doubles) and m, R, I (5),
# write r, v, omega, alpha, q, a (19).
PARTICLE_BYTES_PER_STEP = 344
# Untimed steps before the warm-up, per workload (--preroll overrides).
PREROLL = {"spheres": 3000, "polyhedra": 0, "polyhedra_dense": 0, "drums": 0, "mixer": 300, "polyhedra_mesh": 0,
           "fragments": 0}
# DRAM bytes (read + write) per launch of k_cfused per listed pair and of
# k_fused_epilog per particle, from the ncu capture of the pre-rolled 250k-sphere
# bed (the same workload at 1/8 of its size); they scale with the listed pairs and
# the particles.  Both kernels run their FP64 pipe at the fraction recorded here
# (sm__pipe_fp64_cycles_active of peak sustained).
TRAFFIC = {"source": "profiles/k_cfused_fp64_lanes_spheres_bed_250k.md",
           "contact_bytes_per_listed_pair": 212.0, "epilog_bytes_per_particle": 445.0,
           "contact_fp64_pipe_active": 0.807, "epilog_fp64_pipe_active": 0.820}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default: the workload's whole run, e.g. 1000 for the 2M-sphere deposition)")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--preroll", type=int, default=None,
                    help="untimed steps run before the warm-up (default: the workload's pre-roll, 3000 for the "
                         "spheres; 0 disables)")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain FP64 path leg (vs_plain)")
    ap.add_argument("--patch", type=int, default=125_000,
                    help="spheres: particle count of the periodic patch the CPU legs time (same workload, "
                         "footprint scaled to keep the density)")
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--n", type=int, default=None, help="particle count (default: the workload's)")
    ap.add_argument("--workload", default="spheres",
                    choices=["spheres", "polyhedra", "polyhedra_dense", "drums", "mixer", "polyhedra_mesh",
                             "fragments"],
                    help="spheres: 2M spheres on a floor (headline); polyhedra: 200k polyhedra deposition; "
                         "polyhedra_dense: polyhedra on a dense lattice; drums: 256 rotating drums batched; "
                         "mixer: 50k spheres falling into a mesh (STL) mixer")
    ap.add_argument("--systems", type=int, default=256, help="drums: number of drums")
    ap.add_argument("--plain", action="store_true", help="plain FP64 path (no FP32 screening)")
    ap.add_argument("--no-graph", action="store_true", help="fused step launched from the host, no CUDA graph")
    ap.add_argument("--no-tune", action="store_true", help="skip the autotuner (cell size, launch shapes)")
    ap.add_argument("--mul-mode", type=int, default=None, choices=list(range(8)),
                    help="multiplies on the integer pipe: bit 0 integration rotations, bit 1 integration rest, "
                         "bit 2 contact law (default: the autotuner's choice, else 2)")
    ap.add_argument("--int-share", type=int, default=None, choices=list(range(9)),
                    help="eighths of the fused contact tiles whose law runs on the integer pipe (no effect on "
                         "results; default: the autotuner's choice)")
    ap.add_argument("--cell-broad-phase", action="store_true",
                    help="spheres: the warp-per-cell staged broad phase instead of thread per owner "
                         "(same lists)")
    ap.add_argument("--learned", action="store_true",
                    help="polyhedra: harvest candidate pairs, train the MLP, time with learned sizing "
                         "and without it")
    ap.add_argument("--harvest", type=int, default=5_000_000, help="learned: candidate pairs to harvest")
    ap.add_argument("--learned-mode", type=int, default=1, choices=[1, 2],
                    help="learned: 1 predicted record sizes, 2 also warp bins by predicted contact type")
    ap.add_argument("--epochs", type=int, default=20, help="learned: training epochs")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--rebuild-ms", type=int, default=0,
                    help="after the run, time this many explicit list rebuilds (CUDA events on the library's "
                         "stream); with mesh drivers also on the same particles without the meshes")
    return ap.parse_args()


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            m = json.load(f)
        return float(m["hbm_gbs"]), "measured"
    except Exception:  # noqa: BLE001
        return 6800.0, "fallback"


class Clocks:
    """Samples SM clocks and throttle reasons with nvidia-smi during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, dev_index: int):
        self.dev = dev_index
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except Exception:  # noqa: BLE001
            self.p = None
        return self

    def __exit__(self, *exc):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except Exception:  # noqa: BLE001
                self.p.kill()

    def summary(self):
        try:
            self.f.flush()
            rows = [r.split(",") for r in open(self.f.name).read().strip().splitlines() if r.strip()]
        except Exception:  # noqa: BLE001
            rows = []
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = sorted(float(r[1]) for r in rows)
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for k, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(k)
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": float(rows[0][2]), "reasons": sorted(reasons),
                "samples": len(rows)}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
        return rank, world, local, dist
    return rank, world, local, None


def barrier(dist):
    if dist is not None:
        dist.barrier()


def allmax(dist, x: float) -> float:
    if dist is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def allsum(dist, x: float) -> float:
    if dist is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def workload(args):
    w = _workload(args)
    if args.steps is None:
        args.steps = int(w.steps)
    return w


def _workload(args):
    from exadem_gb300 import workloads as W

    opt = 0 if args.plain else 1
    flags = dict(fp32_contact_screen=opt, fused_step=opt, fp32_broad_phase=opt)
    if args.workload in ("spheres", "drums", "mixer"):
        flags["graph_step"] = opt and not args.no_graph
    if args.learned and args.workload in ("polyhedra", "polyhedra_dense"):
        flags["learned_sizing"] = args.learned_mode
    if args.workload == "polyhedra":
        return W.polyhedra_floor(n=args.n or 200_000, **flags)
    if args.workload == "polyhedra_dense":
        side = round((args.n or 200_000) ** (1.0 / 3.0))
        return W.polyhedra_lattice(nx=side, ny=side, nz=side, **flags)
    if args.workload == "drums":
        return W.drums_batch(nsys=args.systems, nmax=args.n or 200_000, **flags)
    if args.workload == "mixer":
        return W.spheres_mixer(n=args.n, **flags)
    if args.workload == "fragments":
        return W.fragment_blocks(nblocks=max(1, round((args.n or 128_000) / 125)), nx=5, ny=5, nz=5, seed=5,
                                 steps=400, **flags)
    if args.workload == "polyhedra_mesh":
        side = round(((args.n or 4800) / 3) ** 0.5)
        return W.polyhedra_mesh_terrain(nx=side, ny=side, nz=3, amp=0.5, waves=6, m=60, **flags)
    n = args.n or 2_000_000  # a smaller count keeps the density: the footprint scales with it
    return W.spheres_floor(n=n, side=400.0 * math.sqrt(n / 2_000_000), **flags)


def is_batch(w) -> bool:
    return hasattr(w, "members")


def build_from_host(w, arrays):
    """The workload's System, with the particle arrays `arrays` (host buffers)."""
    from exadem_gb300 import System

    s = System(w.params)
    if is_batch(w):
        s.set_particles(arrays)
        for m in w.members:
            for kw in m.surfaces:
                s.register_surface(**kw)
            for kw in m.cylinders:
                s.register_cylinder(**kw)
        s.set_systems(w.systems())
        return s
    if w.shapes:
        s.set_shapes(w.shapes)
    for kw in w.surfaces:
        s.register_surface(**kw)
    for kw in w.cylinders:
        s.register_cylinder(**kw)
    for kw in w.meshes:
        s.register_mesh(**kw)
    s.set_particles(arrays)
    if w.bonds:
        s.set_inner_bond_params(w.bonds["params"])
        s.stick_polyhedra(arrays["id"], w.bonds["cluster"], w.bonds["threshold"])
    return s


WORKLOAD_DESC = {
    "spheres": "spheres_floor: 2M polydisperse spheres r~U[0.4,0.6], periodic x/y, floor wall, "
               "Hooke+cohesion(kc=1e3,dncut=0.01)+kr=100, dt=5e-4",
    "polyhedra": "polyhedra_floor: 200k cubes/tetrahedra/octahedra (Minkowski 0.01), RSA of circumscribed "
                 "spheres at 0.35, floor + side walls, Hooke kn=1e5 kt=8e4 mu=0.5, dt=1e-4",
    "polyhedra_dense": "polyhedra_lattice: cubes/tetrahedra/octahedra on a lattice of spacing 1.3, random "
                       "orientations, Hooke kn=1e4, dt=1e-4",
    "drums": "drums_batch: 256 rotating drums (spheres r~U[0.45,0.55], counts log-uniform in [2e3, 2e5], "
             "30% fill, 2 rad/s, periodic along the axis), Hooke kn=1e4 kt=8e3 mu=0.4, dt=5e-4",
    "polyhedra_mesh": "polyhedra_mesh_terrain: 4800 cubes/tetrahedra/octahedra (40 x 40 x 3 lattice) falling on "
                      "a 7200-triangle terrain mesh (Minkowski 0.02) inside four walls, Hooke kn=1e4, dt=5e-4",
    "fragments": "fragment_blocks: 1024 blocks of 5 x 5 x 5 unit cubes (Minkowski 0.01), face-bonded per block by "
                 "stick_polyhedra (1.2M bonds, 307k interfaces; kn=1e4 kt=8e3 damp 0.87, mixed mode g=0.05), "
                 "turned and falling at 3 m/s onto a floor; Hooke kn=1e5 kt=8e4 mu=0.3, dt=1e-4",
    "mixer": "spheres_mixer: 50,304 spheres r=2 (SC lattice 4.1 in a cylinder r=92) falling into a mesh mixer "
             "(wall, bottom, 4 blades: 2064 triangles, Minkowski 0.1), Hooke kn=1e3 kt=1e3 mu=0.5, dt=1e-3",
}


def cpu_sample(args, w, max_steps: int, budget_s: float):
    """The oracle (C++ restatement of the reference CPU path, OpenMP, all host
    cores) on a bounded sample of the workload.  Spheres: a periodic patch of
    the same workload (args.patch spheres, footprint scaled to keep the density,
    same generator and physics), pre-rolled like the GPU legs, then timed for up
    to max_steps steps or budget_s seconds.  Other workloads: the workload itself
    (one drum at a time for the batched drums), without pre-roll."""
    import math as _m

    from exadem_gb300 import workloads as W
    from oracle.oracle import oracle_system, set_threads

    cores = set_threads(os.cpu_count() or 1)
    if is_batch(w):  # the drums one after another (the oracle runs one system per context)
        done = 0.0
        t_all = 0.0
        nd = 0
        for m in w.members:
            o = m.build(oracle_system)
            o.first_iteration()
            t0 = time.perf_counter()
            o.step(10)
            t_all += time.perf_counter() - t0
            done += m.n * 10
            nd += 1
            o.close()
            if t_all > budget_s:
                break
        return {"value": done / t_all, "unit": UNIT, "cores": cores, "kind": "port", "steps": 10,
                "seconds": t_all,
                "sample": f"10 Verlet steps of each of the first {nd} drums ({int(done / 10)} spheres), "
                          f"{t_all:.1f} s"}
    pre = preroll_steps(args)
    if args.workload == "spheres":
        n = min(args.patch, w.n)
        side = 400.0 * _m.sqrt(n / 2_000_000)
        ws = W.spheres_floor(n=n, side=side)
        what = f"periodic {side:.1f} x {side:.1f} patch of the same workload ({n} spheres)"
    else:
        ws, n, pre = w, w.n, 0
        what = f"the full {w.n}-particle workload"
    o = ws.build(oracle_system)
    t0 = time.perf_counter()
    o.first_iteration()
    if pre:
        o.step(pre)
    o.step(max(1, min(args.warmup, 3)))
    t_pre = time.perf_counter() - t0
    r0 = o.rebuild_count()
    steps = 0
    t0 = time.perf_counter()
    while True:
        o.step(1)
        steps += 1
        el = time.perf_counter() - t0
        if el > budget_s or steps >= max_steps:
            break
    rebuilds = o.rebuild_count() - r0
    o.close()
    return {"value": n * steps / el, "unit": UNIT, "cores": cores, "kind": "port", "steps": steps, "seconds": el,
            "sample": f"{steps} Verlet steps ({rebuilds} rebuilds) of a {what}, after first_iteration, "
                      f"{pre} pre-roll steps and the warm-up ({t_pre:.1f} s, untimed); {el:.1f} s timed"}


def cpu_baseline(args, w):
    return cpu_sample(args, w, max_steps=50, budget_s=20.0)


def run_drums_separate(args, w, rank, world, local, dist):
    """Own plain FP64 GPU path on the batched workload: one context per drum,
    plain operator kernels, the drums stepped one after another (each dem_step
    ends with a stream synchronisation).  Wall-clock timing of the K steps."""
    import torch

    systems = [m.build() for m in w.members]
    for s in systems:
        s.first_iteration()
        s.step(args.warmup)
        s.reset_kernel_stats()
    torch.cuda.synchronize()
    with Clocks(local) as clk:
        barrier(dist)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            for s in systems:
                s.step(1)
        torch.cuda.synchronize()
        el = time.perf_counter() - t0
        barrier(dist)
    launches = sum(sum(v["launches"] for v in s.kernel_stats().values()) for s in systems)
    rebuilds = sum(s.rebuild_count() for s in systems)
    for s in systems:
        s.close()
    el = allmax(dist, el)
    total = allsum(dist, float(w.n * args.steps))
    line = {"metric": METRIC, "value": total / el, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": el * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded random sequential addition)",
            "config": {"workload": WORKLOAD_DESC["drums"] if args.n is None and args.systems == 256 else
                       f"drums n_systems={args.systems} nmax={args.n or 200000}", "n_particles": w.n,
                       "path": "plain FP64 operator kernels, one context per drum, drums stepped in turn",
                       "timing": "wall clock around K steps of all drums, synchronised on both sides",
                       "parallelism": "replicas" if world > 1 else "single"},
            "gpu_launches": launches, "rebuilds_total": rebuilds, "clocks": clk.summary()}
    if rank == 0:
        print(json.dumps(line))


def train_learned(args):
    """Harvests candidate polyhedron pairs with their exact contact counts from
    forced rebuilds of the dense lattice (config 3's shapes and contact law),
    trains the MLP on the GPU, and returns its parameters and a summary."""
    import torch

    from exadem_gb300 import workloads as W
    from exadem_gb300.learned import Learned

    side = round((args.n or 200_000) ** (1.0 / 3.0))
    s = W.polyhedra_lattice(nx=side, ny=side, nz=side, seed=41, fused_step=1, fp32_broad_phase=1,
                            fp32_contact_screen=1).build()
    s.first_iteration()
    L = Learned(s)
    xs, ys, rebuilds = [], [], 0
    t0 = time.perf_counter()
    while sum(x.shape[0] for x in xs) < args.harvest and rebuilds < 40:
        s.update_particle_neighbors()
        x, y, _ = L.harvest(1 << 24)
        xs.append(x.clone())
        ys.append(y.clone())
        rebuilds += 1
        s.step(25)
    x = torch.cat(xs)[: args.harvest].contiguous()
    y = torch.cat(ys)[: args.harvest].contiguous()
    t_harvest = time.perf_counter() - t0
    L.init(seed=4, label_means=y.float().mean(0).tolist())
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    losses = L.train(x, y, epochs=args.epochs, batch=65536, lr=1e-3, seed=4)
    t_train = time.perf_counter() - t0
    rates = L.rates(x)
    tot = y.float().sum(1)
    corr = float(torch.corrcoef(torch.stack([rates.sum(1), tot]))[0, 1])
    params = L.params()
    s.close()
    return params, {"samples": int(x.shape[0]), "harvest_rebuilds": rebuilds, "harvest_s": round(t_harvest, 2),
                    "epochs": args.epochs, "batch": 65536, "lr": 1e-3, "train_s": round(t_train, 2),
                    "loss_first_epoch": losses[0], "loss_last_epoch": losses[-1],
                    "corr_total_count": round(corr, 4),
                    "label_means": [round(v, 4) for v in y.float().mean(0).tolist()]}


def rebuild_timing(args, w, s):
    """Time of one explicit list rebuild in the state the run ended in; with mesh
    drivers, also on the same particles in a system without the meshes."""
    import numpy as np
    import torch

    def timed(sys_):
        ext = torch.cuda.ExternalStream(sys_.stream_handle())
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        for _ in range(args.rebuild_ms):
            sys_.update_particle_neighbors()
        e1.record(ext)
        e1.synchronize()
        return e0.elapsed_time(e1) / args.rebuild_ms

    out = {"rebuilds_timed": args.rebuild_ms, "rebuild_ms": timed(s)}
    if getattr(w, "meshes", None):
        p = s.particles(sort_by_id=True)
        w2 = workload(args)
        w2.meshes = []
        w2.particles = {k: np.ascontiguousarray(v) for k, v in p.items() if k in w2.particles}
        s2 = w2.build()
        s2.first_iteration()
        out["rebuild_ms_without_meshes"] = timed(s2)
        s2.close()
    return out


def preroll_steps(args) -> int:
    return PREROLL.get(args.workload, 0) if args.preroll is None else max(0, args.preroll)


def plain_variant(w):
    """The same workload (same particles, drivers and physics) on the plain FP64
    operator kernels: no fused step, no FP32 screening, no graph, no learned sizing."""
    import copy

    from exadem_gb300 import _abi as A

    q = A.Params.from_buffer_copy(w.params)
    q.fp32_broad_phase = q.fp32_contact_screen = q.fused_step = q.graph_step = q.learned_sizing = 0
    w2 = copy.copy(w)
    w2.params = q
    return w2


def event_timed(s, steps: int, local: int, dist):
    """K steps timed with CUDA events on the library's stream, barrier and synchronise on both sides."""
    import torch

    ext = torch.cuda.ExternalStream(s.stream_handle())
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    r0 = s.rebuild_count()
    with Clocks(local) as clk:
        barrier(dist)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push("timed")  # lets a profiler select the timed steps (ncu --nvtx-include timed/)
        ev0.record(ext)
        s.step(steps)
        ev1.record(ext)
        ev1.synchronize()
        torch.cuda.nvtx.range_pop()
        torch.cuda.synchronize()
        barrier(dist)
    return ev0.elapsed_time(ev1), s.rebuild_count() - r0, clk.summary()


def bed_fraction(s, w) -> dict:
    """Solid fraction of the spheres' bed: the packing profile (analytic sphere-slab
    volumes, 50 slabs from the floor to the highest centre) and its mean over the
    slabs between two diameters above the floor and two diameters below the top."""
    import numpy as np

    p = s.particles(sort_by_id=False)
    zmax = float(np.max(p["rz"]))
    rmax = float(np.max(p["radius"]))
    prof = s.packing_profile(50, 0.0, zmax)
    dz = zmax / 50
    lo, hi = int(np.ceil(2 * rmax / dz)), int(np.floor((zmax - 2 * rmax) / dz))
    core = prof[lo:hi] if hi > lo else prof
    return {"phi_bed": round(float(np.mean(core)), 4), "phi_profile_max": round(float(np.max(prof)), 4),
            "bed_top": round(zmax, 3)}


def run_native(args, rank, world, local, dist):
    import numpy as np
    import torch

    from exadem_gb300 import build as B

    B.build()
    torch.cuda.set_device(local)
    w = workload(args)
    if is_batch(w) and args.plain:
        return run_drums_separate(args, w, rank, world, local, dist)
    pre = preroll_steps(args)
    learned = None
    if args.learned and args.workload in ("polyhedra", "polyhedra_dense"):
        params, learned = train_learned(args)
    s = w.build()
    if learned is not None:
        from exadem_gb300.learned import Learned

        Learned(s).set_params(params)
    s.first_iteration()
    t0 = time.perf_counter()
    if pre:
        s.step(pre)
        torch.cuda.synchronize()
    preroll_s = time.perf_counter() - t0
    state_pre = s.simulation_state()
    # the pre-rolled particle state, read back for the end-to-end leg
    host_pre = None if (args.no_e2e or is_batch(w)) else s.particles(sort_by_id=True)
    bed = bed_fraction(s, w) if args.workload == "spheres" and pre else None
    tune = None
    if not args.plain and not args.no_tune and args.workload in ("spheres", "drums", "mixer"):
        # cell size and launch shapes; the skin only where it cannot change a bit.
        # The mixer's spheres start slow and then fall: the rebuild interval the
        # tuner models from the speeds at the start does not hold, so its skin
        # stays the deck's (rcut_inc 1.2)
        tune = s.autotune(steps_per_trial=3, skin_policy=0 if args.workload == "mixer" else 1)
    if args.mul_mode is not None:
        s.set_mul_mode(args.mul_mode)
    if args.int_share is not None:
        s.set_contact_int_share(args.int_share)
    if args.cell_broad_phase:
        s.set_sphere_cell_broad_phase(1)
    s.step(args.warmup)
    torch.cuda.synchronize()
    s.reset_kernel_stats()
    ms, rebuilds, clocks = event_timed(s, args.steps, local, dist)
    if learned is not None:
        from exadem_gb300.learned import Learned

        learned["last_rebuild"] = Learned(s).stats()
        # the same step without the learned part (the exact two-pass sizing)
        w0 = workload(argparse.Namespace(**{**vars(args), "learned": False}))
        s0 = w0.build()
        s0.first_iteration()
        s0.step(pre + args.warmup)
        ms0, _, _ = event_timed(s0, args.steps, local, None)
        learned["ms_per_step_without"] = ms0 / args.steps
        learned["ms_per_step_with"] = ms / args.steps
        learned["rebuilds_without"] = s0.rebuild_count()
        learned["same_state"] = bool(s0.simulation_state()["kinetic_energy"].tolist()
                                     == s.simulation_state()["kinetic_energy"].tolist())
        s0.close()
    stats = s.kernel_stats()
    launches = sum(v["launches"] for v in stats.values())
    ms = allmax(dist, ms)
    total = allsum(dist, float(w.n * args.steps))
    value = total / (ms / 1e3)
    state_end = s.simulation_state()

    # the plain FP64 operator path from the same initial state, same pre-roll and
    # warm-up: its speed, and whether it ends in the same bits
    vs_plain = None
    if not args.plain and not args.no_plain and not is_batch(w):
        sp = plain_variant(w).build()
        sp.first_iteration()
        sp.step(pre + args.warmup)
        torch.cuda.synchronize()
        msp, rebp, _ = event_timed(sp, args.steps, local, dist)
        a, b = s.particles(sort_by_id=True), sp.particles(sort_by_id=True)
        same = all(np.array_equal(np.ascontiguousarray(a[k]).view(np.uint8), np.ascontiguousarray(b[k]).view(np.uint8))
                   for k in a)
        msp = allmax(dist, msp)
        vs_plain = {"value": total / (msp / 1e3), "unit": UNIT, "ms_per_step": msp / args.steps,
                    "ratio": msp / ms, "rebuilds_in_timed_region": rebp, "same_bits": bool(same),
                    "path": "plain FP64 operator kernels (one kernel per reference operator, exact two-pass "
                            "lists, no FP32 screening, no graph), same pre-roll and warm-up"}
        del a, b
        sp.close()

    # particles whose epilog rotation is exactly zero (no spin, no torque) at the end of the timed run
    pp = s.particles(sort_by_id=False)
    idle = np.ones(w.n, dtype=bool)
    for k in ("vrotx", "vroty", "vrotz", "momx", "momy", "momz"):
        idle &= pp[k].view(np.uint64) == 0
    idle_fraction = float(idle.mean()) if w.n else 0.0
    del pp

    # per-kernel times (profiled run, separate from the timed one)
    s.reset_kernel_stats()
    s.profile(True)
    kprof_steps = max(20, args.steps // 4)
    ni0 = s.interaction_count()
    s.step(kprof_steps)
    prof = s.kernel_stats()
    s.profile(False)
    ni = (ni0 + s.interaction_count()) // 2
    peak, peak_kind = peaks()

    def per_step(keys):
        return sum(prof[k]["total_ms"] for k in keys if k in prof) / kprof_steps / 1e3

    def per_launch(key):
        v = prof.get(key)
        return v["total_ms"] / max(v["timed"], 1) / 1e3 if v else 0.0

    step_ms_prof = sum(v["total_ms"] for v in prof.values()) / kprof_steps
    tot_ms = max(sum(x["total_ms"] for x in prof.values()), 1e-9)
    shares = {k: round(v["total_ms"] / tot_ms, 4) for k, v in prof.items() if v["total_ms"] > 0}
    # the dominant kernel: the contact law over the listed pairs ("contact" is k_cfused when
    # detection and law are fused, k_chooke when they are separate, the whole plain kernel otherwise)
    ran = lambda k: prof.get(k, {}).get("total_ms", 0.0) > 0.0
    fused_contact = ran("contact_screen") and not ran("contact_detect")
    t_law = per_launch("contact")
    achieved_c = CONTACT_BYTES_PER_INTERACTION * ni / t_law / 1e9 if t_law > 0 else 0.0
    t_c = TRAFFIC["contact_bytes_per_listed_pair"] if fused_contact else None
    roofline = {"bound": "hbm",
                "kernel": ("k_cfused (contact detection + contact law over the listed pairs)" if fused_contact
                           else "contact law kernel over the listed pairs"),
                "achieved": achieved_c, "peak": peak, "unit": "GB/s", "frac": achieved_c / peak,
                "peak_kind": peak_kind, "traffic": (t_c * ni if t_c else None),
                "algorithmic_bytes_per_launch": CONTACT_BYTES_PER_INTERACTION * ni, "listed_pairs": ni,
                "algorithmic_bytes_per_unit": CONTACT_BYTES_PER_INTERACTION, "avg_launch_ms": t_law * 1e3,
                "share_of_step": shares.get("contact", 0.0),
                "traffic_source": TRAFFIC["source"] if fused_contact else None,
                "traffic_scaling": ("212 B per listed pair measured at 250k spheres (826k listed pairs), "
                                    "times the listed pairs here") if fused_contact else None,
                "fp64_pipe_active": TRAFFIC["contact_fp64_pipe_active"] if fused_contact else None,
                "note": "FP64-pipe bound, not HBM bound: the FP64 pipe runs at the fp64_pipe_active fraction of "
                        "its peak (2 FP64 instructions per cycle per SM)"}
    t_integ = per_step(("prolog", "epilog"))
    achieved_i = PARTICLE_BYTES_PER_STEP * w.n / t_integ / 1e9 if t_integ > 0 else 0.0
    t_e = TRAFFIC["epilog_bytes_per_particle"]
    roofline_integration = {
        "bound": "hbm", "kernel": "integration (k_fused_prolog + k_fused_epilog + rotation kernels)",
        "achieved": achieved_i, "peak": peak, "unit": "GB/s", "frac": achieved_i / peak, "peak_kind": peak_kind,
        "epilog_traffic": (t_e * w.n if fused_contact else None),
        "algorithmic_bytes_per_launch": PARTICLE_BYTES_PER_STEP * w.n,
        "avg_launch_ms": t_integ * 1e3, "share_of_step": round(shares.get("prolog", 0) + shares.get("epilog", 0), 4),
        "epilog_fp64_pipe_active": TRAFFIC["epilog_fp64_pipe_active"] if fused_contact else None,
        "note": "344 B per particle-step (prolog and epilog together, per step)"}
    t_contact = sum(per_launch(k) for k in ("contact_screen", "contact_detect", "contact"))
    achieved_p = CONTACT_BYTES_PER_INTERACTION * ni / t_contact / 1e9 if t_contact > 0 else 0.0
    roofline_contact_phase = {"bound": "hbm", "kernel": "contact phase (k_cscreen + contact kernels)",
                              "achieved": achieved_p, "peak": peak, "unit": "GB/s", "frac": achieved_p / peak,
                              "algorithmic_bytes_per_launch": CONTACT_BYTES_PER_INTERACTION * ni,
                              "avg_launch_ms": t_contact * 1e3}
    mul_mode = s.mul_mode()
    rebuild = rebuild_timing(args, w, s) if args.rebuild_ms > 0 else None
    s.close()

    # end to end through the C ABI from pinned host buffers (the pre-rolled state)
    e2e = None
    if not args.no_e2e:
        from exadem_gb300 import System

        pinned = {}
        host = w.particles() if is_batch(w) else host_pre
        for k, v in host.items():
            t = torch.empty(v.shape, dtype=torch.from_numpy(v).dtype, pin_memory=True)
            t.numpy()[:] = v
            pinned[k] = t.numpy()
        out = {k: torch.empty(v.shape, dtype=torch.from_numpy(v).dtype, pin_memory=True).numpy()
               for k, v in host.items()}
        h2d = sum(v.nbytes for v in pinned.values())
        barrier(dist)
        t0 = time.perf_counter()
        s2 = build_from_host(w, pinned)
        s2.first_iteration()
        s2.step(args.steps)
        from exadem_gb300 import _abi as A
        import ctypes as C

        st = A.particles_struct(out, w.n)
        s2._check(s2.b.get_particles(s2.h, C.byref(st), 0), "get_particles")
        el = time.perf_counter() - t0
        d2h = sum(v.nbytes for v in out.values())
        s2.close()
        el = allmax(dist, el)
        e2e = {"value": total / el, "unit": UNIT, "h2d_bytes_per_step": h2d / args.steps,
               "d2h_bytes_per_step": d2h / args.steps,
               "note": "context setup, the pre-rolled particle state uploaded from pinned host memory, "
                       "first_iteration, K steps, final state read back; all timed"}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline(args, w)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded random sequential addition)",
        "config": config_block(args, w, pre, preroll_s, bed, mul_mode, idle_fraction),
        "vs_plain": vs_plain,
        "roofline": roofline, "roofline_integration": roofline_integration,
        "roofline_contact_phase": roofline_contact_phase,
        "autotune": ({k: (round(v, 6) if isinstance(v, float) else v) for k, v in tune.items()}
                     if tune else None),
        "learned": learned,
        "kernel_shares": shares, "profiled_ms_per_step": step_ms_prof,
        "rebuilds_in_timed_region": rebuilds, "gpu_launches": launches,
        "clocks": clocks, "e2e": e2e, "cpu_baseline": cpu,
        "state_after_preroll": {"n_interactions": state_pre["n_interactions"],
                                "n_active": state_pre["n_active_interactions"]},
        "state_after": {"n_interactions": state_end["n_interactions"], "n_active": state_end["n_active_interactions"]},
        "rebuild_timing": rebuild,
    }
    if rank == 0:
        print(json.dumps(line))


def config_block(args, w, pre, preroll_s, bed, mul_mode, idle_fraction):
    cfg = {"workload": WORKLOAD_DESC[args.workload] if args.n is None and args.systems == 256
           else f"{args.workload} n={w.n}",
           "n_particles": w.n,
           "path": "plain FP64 operator kernels" if args.plain else
                   "fused step, FP32 broad phase and contact screen, compacted FP64 contact law, exact fast division"
                   + (", whole step replayed as one CUDA graph" if getattr(w.params, "graph_step", 0) else "")
                   + (f", {w.info['systems']} systems in one context" if is_batch(w) else "")
                   + (", warp-per-cell staged sphere broad phase" if args.cell_broad_phase else ""),
           "preroll_steps": pre, "preroll_s": round(preroll_s, 2),
           "timed_window": f"steps {pre + args.warmup + 1}..{pre + args.warmup + args.steps} after first_iteration",
           "mul_mode": None if args.plain else mul_mode,
           "rotation_idle_fraction_at_end": round(idle_fraction, 4),
           "l2": "inputs larger than L2 (particle state 0.5 GB, interactions > 0.5 GB)",
           "parallelism": "replicas" if args.gpus > 1 else "single",
           "inputs": {k: (round(v, 4) if isinstance(v, float) else v) for k, v in w.info.items() if k != "counts"}}
    if bed:
        cfg["bed"] = {**bed, "phi_target": 0.55,
                      "note": "solid fraction of the bed the pre-roll deposited (the RSA initial state jams "
                              "below 0.38)"}
    return cfg


def run_reference(args, rank, world, local, dist):
    """The reference arm: the oracle (C++ restatement of exaDEM's CPU path,
    pinned function by function against exaDEM's own headers; exaDEM itself
    cannot be built without exaNBody/onika/MPI) on all host cores, timed on a
    bounded sample of the native arm's workload (cpu_sample)."""
    if rank != 0:
        return
    w = workload(args)
    cb = cpu_sample(args, w, max_steps=max(1, args.steps), budget_s=60.0)
    v = cb["value"]
    steps = cb["steps"]
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": steps, "warmup": args.warmup,
            "ms_per_step": cb["seconds"] * 1e3 / steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded random sequential addition)",
            "impl": "reference",
            "config": {"workload": WORKLOAD_DESC[args.workload] if args.n is None and args.systems == 256
                       else f"{args.workload} n={w.n}",
                       "n_particles": w.n, "preroll_steps": preroll_steps(args)},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cb["cores"], "kind": cb["kind"],
                             "sample": cb["sample"]},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    args = parse()
    rank, world, local, dist = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, rank, world, local, dist)
    else:
        run_native(args, rank, world, local, dist)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
