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
SAMPLE_SHAPE = (80, 80, 40)   # CPU sample: 8000 elements per part, same aspect
SAMPLE_PARTS = 32


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--shape", default=None, help="override mesh shape nx,ny,nz")
    ap.add_argument("--nparts", type=int, default=None)
    ap.add_argument("--fp32", type=int, default=None)
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


def cpu_sample_seconds(shape, nparts):
    """Run the oracle's RSB once on the sample mesh; returns wall seconds."""
    from parrsb_gb300 import meshgen
    from oracle import oracle as O
    vtx, xyz = meshgen.box_hex(*shape, jitter=0.1, seed=0)
    t = time.perf_counter()
    rc, part, _, info, _ = O.part_mesh(vtx, xyz, nparts, partitioner=0)
    dt = time.perf_counter() - t
    assert rc == 0
    return dt, info.total_iters


def _levels(p):
    n = 0
    while (1 << n) < p:
        n += 1
    return n


def scale_to_workload(sample_seconds, shape, nparts):
    """Element-levels of the full workload over those of the sample."""
    full = SHAPE[0] * SHAPE[1] * SHAPE[2] * _levels(NPARTS)
    samp = shape[0] * shape[1] * shape[2] * _levels(nparts)
    return sample_seconds * full / samp


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import multiprocessing as mp
    from oracle import oracle as O
    O.build()
    cores = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    times = []
    with ctx.Pool(cores) as pool:
        for step in range(args.warmup + args.steps):
            t = time.perf_counter()
            res = pool.starmap(cpu_sample_seconds, [(SAMPLE_SHAPE, SAMPLE_PARTS)] * cores)
            wall = time.perf_counter() - t
            if step >= args.warmup:
                times.append(wall)
    # `cores` samples in `wall` seconds: throughput of the whole host
    per_sample = statistics.median(times) / cores
    est = scale_to_workload(per_sample, SAMPLE_SHAPE, SAMPLE_PARTS)
    out = {
        "impl": "reference", "metric": METRIC, "value": est, "unit": "s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": statistics.median(times) * 1e3, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "rsb_hex_box_256x256x128_to_1024_parts",
                   "elements": SHAPE[0] * SHAPE[1] * SHAPE[2], "nparts": NPARTS,
                   "l2": "inputs larger than L2"},
        "cpu_baseline": {"value": est, "unit": "s", "cores": cores, "kind": "port",
                         "sample": (f"{cores} concurrent oracle RSB runs of a "
                                    f"{'x'.join(map(str, SAMPLE_SHAPE))} box to "
                                    f"{SAMPLE_PARTS} parts (8000 elements per part), "
                                    "time scaled by elements x bisection levels")},
        "e2e": {"value": est, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
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


def other_rows(P, meshgen, lib, torch, ctypes):
    """RCB / RIB of the 512x512 quad annulus (262,144 elements) to 1024 parts,
    gencon on the same annulus (the reference algorithm's element check
    fails there) and on a 128x128x64 jittered hex box (8.4M corner points);
    device-resident inputs, best of 3 after a warm-up."""
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
    # eigensolve (--fp32 0 runs every vector in FP64)
    os.environ["PARRSB_GPU_FP32"] = str(1 if args.fp32 is None else args.fp32)
    os.environ.setdefault("PARRSB_VERBOSE_LEVEL", "0")
    import parrsb_gb300 as P
    from parrsb_gb300 import meshgen
    from parrsb_gb300.options import ParrsbOptions

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
    if not args.no_e2e:
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
    plain = None
    if not args.no_plain:
        os.environ["PARRSB_GPU_BATCHED"] = "0"
        barrier()
        tp0 = time.perf_counter()
        sp = step_device()
        barrier()
        plain = {"value": max_over_ranks(time.perf_counter() - tp0), "unit": "s",
                 "what": "one step with per-group Lanczos launches (no batching, no graphs)",
                 "lanczos_steps": int(sp.lanczos_iters),
                 "kernel_launches": int(sp.kernel_launches)}
        os.environ["PARRSB_GPU_BATCHED"] = "1"

    # ---- the same step with FP64 vectors: time and the error of the mixed path
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
        extras = other_rows(P, meshgen, lib, torch, ctypes)

    s = stats[-1]
    spmv_ms = sum(x.spmv_ms for x in stats)
    spmv_bytes = sum(x.spmv_bytes for x in stats)
    spmv_launches = sum(x.spmv_launches for x in stats)
    achieved = spmv_bytes / (spmv_ms / 1e3) / 1e9 if spmv_ms > 0 else None
    peak, peak_kind = load_peaks()
    traffic = load_traffic()
    per_launch_bytes = spmv_bytes / spmv_launches if spmv_launches else None
    tr_val = None
    if traffic and per_launch_bytes:
        tr_val = traffic.get("dram_bytes_per_algorithmic_byte", None)
        tr_val = tr_val * per_launch_bytes if tr_val else None
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        from oracle import oracle as O
        O.build()
        dt, _ = cpu_sample_seconds(SAMPLE_SHAPE, SAMPLE_PARTS)
        cpu = {"value": scale_to_workload(dt, SAMPLE_SHAPE, SAMPLE_PARTS), "unit": "s",
               "cores": 1, "kind": "port",
               "sample": (f"oracle RSB of a {'x'.join(map(str, SAMPLE_SHAPE))} box to "
                          f"{SAMPLE_PARTS} parts (8000 elements per part) took {dt:.1f} s; "
                          "scaled by elements x bisection levels")}
    h2d = vtx.nbytes + xyz.nbytes
    out = {
        "metric": METRIC, "value": t_dev, "unit": "s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_dev * 1e3,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64" if os.environ.get("PARRSB_GPU_FP32", "0") == "1" else "f64",
        "data": "synthetic",
        "config": {"workload": f"rsb_hex_box_{'x'.join(map(str, shape))}_to_{nparts}_parts",
                   "elements": nel, "nparts": nparts, "rsb_tol": 1e-5,
                   "rsb_max_iter": 50, "rsb_max_passes": 50, "rsb_pre": "rcb",
                   "batched": "all groups of a level per launch, one CUDA graph per pass",
                   "l2": "inputs (2.1 GB mesh) larger than L2",
                   "parallelism": f"replicas x{world}"},
        "e2e": {"value": t_e2e, "unit": "s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(part.nbytes), "last_call": e2e_stages},
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
                     "algorithmic_bytes_per_launch": per_launch_bytes},
        "cpu_baseline": cpu,
        "plain_gpu": plain,
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
        "lanczos_passes": int(s.lanczos_passes),
    }
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
