"""Benchmark: recursive spectral bisection of an 8,388,608-element jittered
hex box (256 x 256 x 128) into 1024 parts on one GB300.

One step = one full parrsb_part_mesh (RSB, Lanczos, RCB pre-partition,
rsb_tol 1e-5, 50 x 50 iterations) of the synthetic mesh.

  value  seconds per partition with the mesh resident in HBM
         (parrsb_part_mesh_device), CUDA events on the library stream.
  e2e    the same through parrsb_part_mesh with host buffers: the timed
         region includes the H2D copy of vertices and coordinates from pinned
         memory and the D2H copy of the part array every step.

With --gpus N (one process per GPU under torchrun) every rank partitions its
own replica of the mesh (the path does not shard across GPUs); time is the
max over ranks.  --impl reference times the CPU restatement of the
reference's algorithm (the reference itself needs MPI and gslib, which are
not installed) on the host cores.
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

METRIC = "RSB s, 8M hex→1024 parts: warm+batched vs plain GPU, cut±1%, tol 1e-5"
SHAPE = (256, 256, 128)
NPARTS = 1024


def workload_config(shape, nparts):
    """The workload, identical in both arms' lines."""
    return {"workload": f"rsb_hex_box_{'x'.join(map(str, shape))}_to_{nparts}_parts",
            "elements": shape[0] * shape[1] * shape[2], "nparts": nparts, "rsb_tol": 1e-5,
            "rsb_max_iter": 50, "rsb_max_passes": 50, "rsb_pre": "rcb",
            "mesh": "jittered hex box on [0,1]^3, jitter 0.1 h, seed 0",
            "l2": "inputs (2.1 GB mesh) larger than L2"}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--shape", default=None, help="override mesh shape nx,ny,nz")
    ap.add_argument("--nparts", type=int, default=None)
    ap.add_argument("--fp32", type=int, default=None)
    ap.add_argument("--method", default="warm", choices=["warm", "reference", "learned"],
                    help="warm: geometric warm start + residual stop; reference: the "
                         "reference's start vector and stopping rule; learned: the "
                         "learned warm start (network) + residual stop")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer leg")
    ap.add_argument("--no-plain", action="store_true",
                    help="skip the per-group (unbatched) comparison step")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the RCB / RIB / gencon legs")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)["hbm_gbs"], "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def load_traffic():
    """DRAM bytes per algorithmic byte of one SpMV launch, from the committed
    ncu summary of a smaller case (the benchmark's launches are scaled by
    their own algorithmic bytes: traffic grows with the matrix)."""
    path = os.path.join(ROOT, "profiles", "k_spmv_rsb_hex_128x128x64_level0.md")
    try:
        with open(path) as f:
            for line in f:
                if line.startswith("| dram_bytes_per_algorithmic_byte |"):
                    return {"dram_bytes_per_algorithmic_byte": float(line.split("|")[2]),
                            "source": os.path.relpath(path, ROOT)}
    except (OSError, ValueError):
        pass
    return None


def load_fixture(name):
    """Oracle RSB of the workload (tests/golden/make_rsb_fixtures.py)."""
    path = os.path.join(ROOT, "tests", "golden", f"rsb_{name}.json")
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return None


def _levels(p):
    n = 0
    while (1 << n) < p:
        n += 1
    return n


def workload_name(shape, nparts):
    return f"hex_box_{'x'.join(map(str, shape))}_to_{nparts}"


def cpu_level0_seconds(vtx, xyz, nparts, threads):
    """CPU baseline sample: the oracle's first bisection (level 0: RCB
    pre-partition, dual graph, Lanczos, sort, components) of the workload
    itself on `threads` host threads.  Returns (seconds, rows x steps)."""
    from oracle import oracle as O
    O.build()
    O.threads(threads)
    lv = O.RsbLevels(vtx, xyz, nparts)
    t = time.perf_counter()
    lv.level()
    return time.perf_counter() - t, lv.info.row_iters


def run_reference(args):
    """The reference arm: the oracle (CPU restatement of the reference's
    RSB) on the workload itself, on all host threads.  One step is one RSB
    level of the real 8M -> 1024 partition (a bounded sample of the
    workload): steps run the levels in order, one partition after another
    (step s runs level s mod L of partition s div L, its input the previous
    step's output), warm-up steps first.  value = the sum over the L levels
    of each level's median timed time: seconds per whole partition, every
    level measured on its real input.  Levels that no timed step reached
    are run once after the timed region and enter with that time."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle import oracle as O
    from parrsb_gb300 import meshgen
    O.build()
    cores = os.cpu_count() or 1
    O.threads(cores)
    shape = tuple(int(x) for x in args.shape.split(",")) if args.shape else SHAPE
    nparts = args.nparts or NPARTS
    vtx, xyz = meshgen.box_hex(*shape, jitter=0.1, seed=0)
    lv = O.RsbLevels(vtx, xyz, nparts)
    ncuts = lv.ncuts
    fresh = lv.state()
    timed = {L: [] for L in range(ncuts)}
    step_t = []
    quality = None

    def one_level(s):
        nonlocal quality
        L = s % ncuts
        if L == 0:
            lv.restore(fresh)
            lv.info = O.RsbInfo()
        t = time.perf_counter()
        lv.level()
        dt = time.perf_counter() - t
        if L == ncuts - 1 and quality is None:  # first complete partition
            part = lv.part()
            q = O.part_quality(part, vtx, nparts)
            quality = {"weighted_cut": q[0], "imbalance": q[5],
                       "lanczos_steps": int(lv.info.total_iters),
                       "max_fiedler_resid": lv.info.max_resid}
        return L, dt

    s = 0
    for _ in range(args.warmup):
        one_level(s)
        s += 1
    t_all = time.perf_counter()
    for _ in range(args.steps):
        L, dt = one_level(s)
        s += 1
        timed[L].append(dt)
        step_t.append(dt)
    timed_wall = time.perf_counter() - t_all
    untimed = {}
    while any(not timed[L] for L in range(ncuts)) or quality is None:
        L, dt = one_level(s)
        s += 1
        if not timed[L]:
            untimed[L] = dt
    per_level = [statistics.median(timed[L]) if timed[L] else untimed[L] for L in range(ncuts)]
    value = sum(per_level)
    fx = load_fixture(workload_name(shape, nparts))
    quality["equals_fixture"] = bool(fx is not None
                                     and quality["weighted_cut"] == fx["weighted_cut"]
                                     and quality["lanczos_steps"] == fx["lanczos_steps"])
    out = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": statistics.mean(step_t) * 1e3 if step_t else None,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": workload_config(shape, nparts),
        "cpu_baseline": {"value": value, "unit": "s", "cores": cores, "kind": "port",
                         "sample": (f"oracle RSB of the workload itself on {cores} host threads; "
                                    f"one step = one of its {ncuts} levels on that level's real "
                                    "input, levels in order, partition after partition; value = "
                                    "sum of the levels' median step times"
                                    + (f" ({len(untimed)} levels untimed: timed once after the "
                                       "timed region)" if untimed else ""))},
        "e2e": {"value": value, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "timed_region_s": timed_wall,
        "level_s": [round(x, 3) for x in per_level],
        "quality": quality,
    }
    print(json.dumps(out))


def _time_device(fn, reps=3):
    import torch
    fn()
    torch.cuda.synchronize()
    best = None
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        fn()
        b.record()
        torch.cuda.synchronize()
        t = a.elapsed_time(b) / 1e3
        best = t if best is None else min(best, t)
    return best


def other_rows(P, meshgen, lib, torch, ctypes, np):
    """RCB / RIB of the 512x512 quad annulus (262,144 elements) to 1024 parts,
    gencon on the same annulus (the reference algorithm's element check
    fails there) and on a 128x128x64 jittered hex box (8.4M corner points),
    the batched level solve of 4,096 subgraphs, and RSB of the 128x128x64
    annular pipe into 256 parts in both precisions; device-resident inputs,
    best of 3 after a warm-up."""
    from parrsb_gb300.options import ParrsbOptions
    out = {}
    vtx, xyz = meshgen.annulus_quad(512, 512, amp=0.02, seed=0)
    d_xyz = torch.from_numpy(xyz).cuda()
    d_part = torch.empty(len(xyz), dtype=torch.int32, device="cuda")
    for name, pa in (("rcb", 1), ("rib", 2)):
        def run(pa=pa):
            o = ParrsbOptions.make(partitioner=pa, verbose_level=0)
            rc = lib.parrsb_part_mesh_device(ctypes.c_void_p(d_part.data_ptr()), None,
                                             ctypes.c_void_p(d_xyz.data_ptr()), len(xyz), 4,
                                             ctypes.byref(o), 1024)
            assert rc == 0
        t = _time_device(run)
        out[name + "_annulus_512x512_to_1024"] = {"s": t, "elements_per_s": len(xyz) / t}
    d_ids = torch.empty(xyz.shape[0] * 4, dtype=torch.int64, device="cuda")

    def gc2():
        rc = lib.parrsb_conn_mesh_device(ctypes.c_void_p(d_ids.data_ptr()),
                                         ctypes.c_void_p(d_xyz.data_ptr()), len(xyz), 2, 0.2)
        assert rc == 1  # element_check fails, as in the reference algorithm
    t = _time_device(gc2)
    out["gencon_annulus_512x512"] = {"s": t, "return_code": 1,
                                     "distinct_ids": int(P.last_stats().gencon_segments)}
    # batched level solve: 4,096 subgraphs (200-20,000 elements, 5% deleted),
    # the Fiedler vector of every one: one segmented launch sequence per
    # Lanczos pass (CUDA graph) against one subgraph at a time
    vc, _, sc = meshgen.subboxes(4096, smin=200, smax=20000, delete=0.05, seed=0)
    c4 = {"subgraphs": 4096, "elements": int(len(vc))}
    n512 = int(np.searchsorted(sc, 512))
    for mode, batched, ng in (("segmented", True, 4096), ("segmented_first_512", True, 512),
                              ("per_subgraph_first_512", False, 512)):
        n = len(vc) if ng == 4096 else n512
        P.fiedler_groups(vc[:50000], sc[:50000], int(sc[49999]) + 1, batched=batched)  # warm-up
        t = time.perf_counter()
        f, it, rs = P.fiedler_groups(vc[:n], sc[:n], ng, batched=batched)
        st = P.last_stats()
        c4[mode] = {"s": time.perf_counter() - t, "elements": n, "lanczos_steps": int(it.sum()),
                    "kernel_launches": int(st.kernel_launches),
                    "resid_p99": float(np.percentile(rs, 99)), "resid_max": float(rs.max()),
                    "above_tol": int((rs > 1e-5).sum())}
    c4["segmented_speedup_first_512"] = (c4["per_subgraph_first_512"]["s"] /
                                         c4["segmented_first_512"]["s"])
    c4["components_max"] = int(P.components(vc, sc, 4096).max())
    out["c4_batched_level_solve"] = c4
    del vc, sc
    # RSB of the 128x128x64 annular pipe (1,048,576 elements) into 256 parts,
    # FP32 and FP64 Lanczos vectors, the benchmark's method; the oracle's cut
    # of the same input from the committed fixture
    vp, xp = meshgen.pipe_hex(128, 128, 64, jitter=0.05, seed=0)
    dvp, dxp = torch.from_numpy(vp).cuda(), torch.from_numpy(xp).cuda()
    dpp = torch.empty(len(vp), dtype=torch.int32, device="cuda")
    with open(os.path.join(ROOT, "tests", "golden", "rsb_hex_pipe_128x128x64_to_256.json")) as fh:
        fx = json.load(fh)
    c3 = {"elements": int(len(vp)), "nparts": 256, "oracle_weighted_cut": fx["weighted_cut"]}
    saved = os.environ.get("PARRSB_GPU_FP32")
    for name, fp32 in (("fp32", "1"), ("fp64", "0")):
        os.environ["PARRSB_GPU_FP32"] = fp32

        def runp():
            o = ParrsbOptions.make(partitioner=0, verbose_level=0)
            rc = lib.parrsb_part_mesh_device(ctypes.c_void_p(dpp.data_ptr()),
                                             ctypes.c_void_p(dvp.data_ptr()),
                                             ctypes.c_void_p(dxp.data_ptr()), len(vp), 8,
                                             ctypes.byref(o), 256)
            assert rc == 0
        t = _time_device(runp)
        stp = P.last_stats()
        cut = P.part_quality(dpp.cpu().numpy(), vp, 256)[0]
        c3[name] = {"s": t, "weighted_cut": cut, "cut_over_oracle": cut / fx["weighted_cut"],
                    "max_fiedler_resid": stp.max_fiedler_resid,
                    "lanczos_steps": int(stp.lanczos_iters)}
    if saved is None:
        os.environ.pop("PARRSB_GPU_FP32", None)
    else:
        os.environ["PARRSB_GPU_FP32"] = saved
    out["c3_pipe_128x128x64_to_256"] = c3
    del vp, xp, dvp, dxp, dpp
    _, xyz3 = meshgen.box_hex(128, 128, 64, jitter=0.1, seed=0)
    d3 = torch.from_numpy(xyz3).cuda()
    ids3 = torch.empty(xyz3.shape[0] * 8, dtype=torch.int64, device="cuda")

    def gc3():
        rc = lib.parrsb_conn_mesh_device(ctypes.c_void_p(ids3.data_ptr()),
                                         ctypes.c_void_p(d3.data_ptr()), len(xyz3), 3, 0.2)
        assert rc == 0
    t = _time_device(gc3)
    out["gencon_hex_box_128x128x64"] = {"s": t, "points_per_s": xyz3.shape[0] * 8 / t,
                                        "distinct_ids": int(P.last_stats().gencon_segments)}
    return out


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    rank, world, local = dist_env()
    import ctypes

    import numpy as np
    import torch

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    # the named method: FP32 vectors on exact integer weights, FP64 dots and
    # eigensolve (--fp32 0 runs every vector in FP64); warm start: the
    # geometric guess per group, judged against the reference's step start
    # (groups with two nearly equal axes keep the step start); batched: all
    # groups of a level per launch; Lanczos restarts until every Fiedler
    # vector's FP64 eigen-residual is at most rsb_tol (--method reference:
    # the reference's start vector and stopping rule)
    os.environ["PARRSB_GPU_FP32"] = str(1 if args.fp32 is None else args.fp32)
    method_env = ({"PARRSB_GPU_START": "2", "PARRSB_GPU_RESID_STOP": "1"}
                  if args.method in ("warm", "learned") else
                  {"PARRSB_GPU_START": "0", "PARRSB_GPU_RESID_STOP": "0"})
    method_env.update({"PARRSB_GPU_WARM": "1" if args.method == "learned" else "0",
                       "PARRSB_GPU_WARM_MIN": "0"})
    os.environ.update(method_env)
    os.environ.setdefault("PARRSB_VERBOSE_LEVEL", "0")
    import parrsb_gb300 as P
    from parrsb_gb300 import meshgen
    from parrsb_gb300 import warm as W
    from parrsb_gb300.options import ParrsbOptions

    # the shipped warm-start network, read by the library when a call asks
    # for the learned start (PARRSB_GPU_WARM=1)
    warm_ok = os.path.exists(W.WEIGHTS)
    if warm_ok:
        os.environ.setdefault("PARRSB_GPU_WARM_WEIGHTS", W.WEIGHTS)

    shape = tuple(int(x) for x in args.shape.split(",")) if args.shape else SHAPE
    nparts = args.nparts or NPARTS
    nel = shape[0] * shape[1] * shape[2]
    vtx, xyz = meshgen.box_hex(*shape, jitter=0.1, seed=0)
    lib = P.library()
    # pinned host copies (e2e) and device-resident copies (value)
    h_vtx = torch.from_numpy(vtx).pin_memory()
    h_xyz = torch.from_numpy(xyz).pin_memory()
    h_part = torch.empty(nel, dtype=torch.int32).pin_memory()
    d_vtx = h_vtx.cuda()
    d_xyz = h_xyz.cuda()
    d_part = torch.empty(nel, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()

    def opts():
        return ParrsbOptions.make(partitioner=0, verbose_level=0)

    def step_device():
        o = opts()
        rc = lib.parrsb_part_mesh_device(ctypes.c_void_p(d_part.data_ptr()),
                                         ctypes.c_void_p(d_vtx.data_ptr()),
                                         ctypes.c_void_p(d_xyz.data_ptr()), nel, 8,
                                         ctypes.byref(o), nparts)
        assert rc == 0, rc
        return P.last_stats()

    def step_host():
        o = opts()
        rc = lib.parrsb_part_mesh(ctypes.c_void_p(h_part.data_ptr()),
                                  ctypes.c_void_p(h_vtx.data_ptr()),
                                  ctypes.c_void_p(h_xyz.data_ptr()), None, nel, 8,
                                  ctypes.byref(o), nparts)
        assert rc == 0, rc
        return P.last_stats()

    from parrsb_gb300 import replicas

    def barrier():
        replicas.barrier(world)
        torch.cuda.synchronize()

    def max_over_ranks(x):
        return replicas.max_over_ranks(x, world)

    # a user of the host entry point makes its first call before anything
    # else fills the device: the library's cached upload buffers are
    # allocated then (device memory allocated after the stream-ordered pool
    # has grown to tens of GB receives host copies several times slower)
    if not args.no_e2e:
        step_host()
    for _ in range(args.warmup):
        step_device()
    # ---- timed region (device-resident inputs, no per-launch events)
    os.environ["PARRSB_GPU_TIMING"] = "0"
    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    timed = []
    for _ in range(args.steps):
        timed.append(step_device())
    ev1.record()
    barrier()
    clock_info = clocks.stop()
    t_dev = max_over_ranks(ev0.elapsed_time(ev1) / 1e3 / args.steps)
    # ---- one more step with CUDA events around every SpMV and vector update
    # of the Lanczos graphs (per-kernel times for the roofline and breakdown)
    os.environ["PARRSB_GPU_TIMING"] = "1"
    stats = [step_device()]
    os.environ["PARRSB_GPU_TIMING"] = "0"
    # ---- end to end (host buffers, copies inside the timed region)
    t_e2e = None
    e2e_stages = None
    link = None
    if not args.no_e2e:
        # this machine's host-to-device bandwidth from the same pinned buffers
        # into the device copies (the e2e leg's extra time is mostly this)
        lt = []
        for _ in range(4):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            d_vtx.copy_(h_vtx, non_blocking=True)
            d_xyz.copy_(h_xyz, non_blocking=True)
            torch.cuda.synchronize()
            lt.append(time.perf_counter() - t0)
        t_link = statistics.median(lt[1:])
        link = {"h2d_gbs": (vtx.nbytes + xyz.nbytes) / t_link / 1e9,
                "h2d_ms_for_inputs": round(t_link * 1e3, 2)}
        step_host()
        barrier()
        t0 = time.perf_counter()
        per_call = []
        for _ in range(args.steps):
            se = step_host()
            per_call.append((se.stage_ms[0], se.stage_ms[9], se.total_ms,
                             sum(se.stage_ms[1:9])))
        barrier()
        t_e2e = max_over_ranks((time.perf_counter() - t0) / args.steps)
        # where the host-buffer call spends its time, median and max over the
        # timed calls: H2D copy, D2H copy, the whole call (host clock), and
        # the device stages in between
        e2e_stages = {}
        for k, name in enumerate(["upload_ms", "download_ms", "call_ms", "device_stages_ms"]):
            xs = [c[k] for c in per_call]
            e2e_stages[name] = round(statistics.median(xs), 2)
            e2e_stages[name.replace("_ms", "_max_ms")] = round(max(xs), 2)
        part = h_part.numpy().copy()
    else:
        part = d_part.cpu().numpy()
    q = P.part_quality(part, vtx, nparts)
    # ---- plain GPU path: every group of a level solved by its own launches
    # ---- the plain GPU path: the reference's start vector, every group of a
    # level solved by its own launches (no batching, no graphs), the same
    # tolerance and stopping rule
    plain = None
    if not args.no_plain:
        os.environ["PARRSB_GPU_BATCHED"] = "0"
        os.environ["PARRSB_GPU_START"] = "0"
        barrier()
        tp0 = time.perf_counter()
        sp = step_device()
        barrier()
        plain = {"value": max_over_ranks(time.perf_counter() - tp0), "unit": "s",
                 "what": ("one step with the reference's start vector and per-group Lanczos "
                          "launches (no batching, no graphs), same stopping rule"),
                 "lanczos_steps": int(sp.lanczos_iters),
                 "max_fiedler_resid": sp.max_fiedler_resid,
                 "weighted_cut": P.part_quality(d_part.cpu().numpy(), vtx, nparts)[0],
                 "kernel_launches": int(sp.kernel_launches)}
        os.environ.update(method_env)
        os.environ["PARRSB_GPU_BATCHED"] = "1"

    # ---- the same step with FP64 vectors: time and the error of the mixed path
    # ---- start vectors and stopping rules, one step each on the same mesh:
    # the reference's step start, the learned start (judged per group), a
    # random start; the reference's stopping rule, and restarts until the
    # eigen-residual is at most rsb_tol
    starts = None
    if not args.no_plain:
        starts = {}
        def leg(start, stop, warm=0, warm_min=0, reorth=0):
            return {"PARRSB_GPU_START": str(start), "PARRSB_GPU_RESID_STOP": str(stop),
                    "PARRSB_GPU_WARM": str(warm), "PARRSB_GPU_WARM_MIN": str(warm_min),
                    "PARRSB_GPU_REORTH": str(reorth)}
        legs = [("reference_start", leg(0, 0)), ("random_start", leg(1, 0)),
                ("geometric_start", leg(2, 0)),
                ("reference_start_resid_stop", leg(0, 1)),
                ("geometric_start_resid_stop", leg(2, 1)),
                ("geometric_start_resid_stop_reorth", leg(2, 1, reorth=1)),
                ("reference_start_reorth", leg(0, 0, reorth=1))]
        if warm_ok:
            legs += [("learned_start", leg(0, 0, 1)),
                     ("learned_start_resid_stop", leg(0, 1, 1)),
                     ("learned_1M_geometric_resid_stop", leg(2, 1, 1, 1 << 20))]
        for name, env in legs:
            saved = {k: os.environ.get(k) for k in env}
            os.environ.update(env)
            try:
                step_device()  # warm-up of this leg's kernels and graphs
                barrier()
                ta, tb = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                ta.record()
                sl = step_device()
                tb.record()
                barrier()
                ql = P.part_quality(d_part.cpu().numpy(), vtx, nparts)
                starts[name] = {
                    "s": max_over_ranks(ta.elapsed_time(tb) / 1e3),
                    "lanczos_steps": int(sl.lanczos_iters), "passes": int(sl.lanczos_passes),
                    "weighted_cut": ql[0], "imbalance": ql[5],
                    "max_fiedler_resid": sl.max_fiedler_resid,
                    "unconverged": int(sl.unconverged),
                    "warm_groups": [int(sl.warm_used), int(sl.warm_tried)],
                    "warm_inference_ms": round(sl.warm_ms, 2),
                    "start_resid": [sl.start_resid_fallback, sl.start_resid_warm],
                    "level_steps": [int(x) for x in sl.level_steps[:int(sl.levels)]]}
            finally:
                for k, v in saved.items():
                    if v is None:
                        os.environ.pop(k, None)
                    else:
                        os.environ[k] = v

    fp64 = None
    if not args.no_plain and os.environ["PARRSB_GPU_FP32"] == "1":
        os.environ["PARRSB_GPU_FP32"] = "0"
        step_device()  # warm-up of the FP64 kernels
        barrier()
        tf0 = time.perf_counter()
        s64 = step_device()
        barrier()
        t64 = max_over_ranks(time.perf_counter() - tf0)
        q64 = P.part_quality(d_part.cpu().numpy(), vtx, nparts)
        fp64 = {"value": t64, "unit": "s", "what": "one step, every Lanczos vector in FP64",
                "weighted_cut": q64[0], "imbalance": q64[5],
                "cut_mixed_over_fp64": q[0] / q64[0] if q64[0] else None,
                "max_fiedler_resid": s64.max_fiedler_resid}
        os.environ["PARRSB_GPU_FP32"] = "1"

    extras = None
    if not args.no_extras and rank == 0:
        extras = other_rows(P, meshgen, lib, torch, ctypes, np)

    s = stats[-1]
    spmv_ms = sum(x.spmv_ms for x in stats)
    spmv_bytes = sum(x.spmv_bytes for x in stats)
    spmv_launches = sum(x.spmv_launches for x in stats)
    achieved = spmv_bytes / (spmv_ms / 1e3) / 1e9 if spmv_ms > 0 else None
    peak, peak_kind = load_peaks()
    traffic = load_traffic()
    per_launch_bytes = spmv_bytes / spmv_launches if spmv_launches else None
    # the whole pass graph: SpMV bytes plus the vector updates' 3 x 4 B per
    # row and step each (FP32), over the pass graphs' device time
    vec_bytes = 2 * 3 * 4 * sum(x.lanczos_row_iters for x in stats)
    pass_ms = sum(x.lanczos_ms[5] for x in stats)
    pass_gbs = (spmv_bytes + vec_bytes) / (pass_ms / 1e3) / 1e9 if pass_ms > 0 else None
    tr_val = None
    if traffic and per_launch_bytes:
        tr_val = traffic.get("dram_bytes_per_algorithmic_byte", None)
        tr_val = tr_val * per_launch_bytes if tr_val else None
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        # the first bisection of this workload on all host threads, scaled to
        # the whole partition by the oracle's own rows x Lanczos steps per
        # level (committed fixture of the full oracle run)
        threads = os.cpu_count() or 1
        dt, rows0 = cpu_level0_seconds(vtx, xyz, nparts, threads)
        fx = load_fixture(workload_name(shape, nparts))
        if fx and fx["levels"] and fx["levels"][0]["row_steps"] == rows0:
            scale = fx["row_steps"] / rows0
            how = (f"level 0 of this workload took {dt:.2f} s; scaled by the oracle's rows x "
                   f"Lanczos steps of all levels over level 0's ({scale:.2f}, fixture "
                   f"tests/golden/rsb_{workload_name(shape, nparts)}.json)")
        else:
            scale = float(_levels(nparts))
            how = (f"level 0 of this workload took {dt:.2f} s; scaled by the number of "
                   f"levels ({scale:.0f}); no matching fixture")
        cpu = {"value": dt * scale, "unit": "s", "cores": threads, "kind": "port",
               "sample": how}
    h2d = vtx.nbytes + xyz.nbytes
    out = {
        "metric": METRIC, "value": t_dev, "unit": "s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_dev * 1e3,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64" if os.environ.get("PARRSB_GPU_FP32", "0") == "1" else "f64",
        "data": "synthetic",
        "config": workload_config(shape, nparts),
        "method": {"batched": "all groups of a level per launch, one CUDA graph per pass",
                   "start": ("geometric warm start -sin(pi x1/2) along each group's principal "
                             "axis in element spacings, judged per group against the "
                             "reference's step start by FP64 eigen-residual; groups with two "
                             "axes within 5% take it along RCB's cut axis"
                             if args.method == "warm" else
                             "learned warm start (network), judged per group the same way"
                             if args.method == "learned" else "the reference's step start"),
                   "stop": ("restart until the FP64 eigen-residual <= rsb_tol; a pass "
                            "ends once its Ritz residual bound (checked after steps 3, 6, "
                            "9, ...) is below 0.7 rsb_tol"
                            if args.method in ("warm", "learned") else
                            "the reference's CG-residual rule"),
                   "learned_start": "see start_vectors.learned_* (network inference cost "
                                    "included)",
                   "env": method_env, "parallelism": f"replicas x{world}"},
        "e2e": {"value": t_e2e, "unit": "s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(part.nbytes), "last_call": e2e_stages,
                "link": link},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None,
                     "traffic": tr_val, "kernel": "k_spmv (sliced-ELL Laplacian)",
                     "traffic_note": ("DRAM bytes per launch: ncu dram bytes / algorithmic "
                                      "bytes of one level-0 launch on the 1M-element box "
                                      f"({traffic['dram_bytes_per_algorithmic_byte']:.3f}, "
                                      f"{traffic['source']}) x this launch's algorithmic "
                                      "bytes") if traffic else None,
                     "peak_source": f"{peak_kind} hbm_gbs",
                     "spmv_ms_per_launch": spmv_ms / spmv_launches if spmv_launches else None,
                     "timed_on": "one step after the timed region, CUDA events around every "
                                 "SpMV launch inside the Lanczos graphs",
                     "algorithmic_bytes_per_launch": per_launch_bytes,
                     "pass_graphs": {"achieved": pass_gbs,
                                     "frac": (pass_gbs / peak) if pass_gbs else None,
                                     "what": ("SpMV plus P / R update bytes of every Lanczos "
                                              "step over the pass graphs' device time "
                                              "(eigensolves, Ritz vectors, finalisations "
                                              "and residual checks included)")}},
        "cpu_baseline": cpu,
        "plain_gpu": plain,
        "start_vectors": starts,
        "fp64_gpu": fp64,
        "other_rows": extras,
        "clocks": clock_info,
        "gpu_launches": int(sum(x.kernel_launches for x in timed)),
        "elements_per_s": nel / t_dev,
        "quality": {"weighted_cut": q[0], "cut_pairs": q[1], "imbalance": q[5],
                    "comm_volume": q[6]},
        "lanczos_steps": int(s.lanczos_iters), "max_fiedler_resid": s.max_fiedler_resid,
        "spmv_launches_per_step": int(s.spmv_launches),
        "unconverged_bisections": int(s.unconverged), "levels": int(s.levels),
        "stage_ms": dict(zip(P.STAGES, [round(x, 2) for x in s.stage_ms])),
        "lanczos_breakdown_ms": dict(zip(["p_update", "r_update", "eigensolve", "ritz",
                                          "pass_setup", "pass_device_total"],
                                         [round(x / len(stats), 2) for x in
                                          [sum(st.lanczos_ms[i] for st in stats)
                                           for i in range(6)]])),
        "lanczos_spmv_ms": round(spmv_ms / len(stats), 2),
        "lanczos_host_ms": dict(zip(["start_vectors", "graph_capture", "restart_loop",
                                     "residual_check"],
                                    [round(x, 2) for x in timed[-1].lanczos_host_ms])),
        "lanczos_passes": int(s.lanczos_passes),
    }
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
