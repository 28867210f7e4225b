"""Writes tests/golden/rsb_<name>.json: the oracle's RSB of the two large
seeded workloads, for the GPU parity tests and the benchmark.

  hex_box_256x256x128_to_1024  8,388,608 jittered hex elements (seed 0,
                               jitter 0.1 h) into 1024 parts
  hex_pipe_128x128x64_to_256   1,048,576 hex elements of an annular
                               cylinder (seed 0, jitter 0.05 h) into 256 parts

Both with the reference's defaults: Lanczos (rsb_algo 0), RCB
pre-partition, rsb_tol 1e-5, 50 steps x 50 restarts, component counts on.
Each fixture records the mesh's SHA-256 (vertex ids and coordinates; the
pipe uses sin / cos, whose last bits may differ between platforms), the
partition's quality figures, part sizes by part number, the SHA-256 of the
part array, and Lanczos steps per level.  The oracle runs one level at a
time on all host threads (the result does not depend on the thread count).

    python tests/golden/make_rsb_fixtures.py [box|pipe|all]
"""
import hashlib
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "box": ("hex_box_256x256x128_to_1024", "box_hex", (256, 256, 128), {"jitter": 0.1, "seed": 0},
            1024),
    "pipe": ("hex_pipe_128x128x64_to_256", "pipe_hex", (128, 128, 64),
             {"jitter": 0.05, "seed": 0}, 256),
}


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def make_mesh(kind):
    from parrsb_gb300 import meshgen
    name, gen, shape, kw, nparts = WORKLOADS[kind]
    vtx, xyz = getattr(meshgen, gen)(*shape, **kw)
    return name, vtx, xyz, nparts


def run(kind):
    from oracle import oracle as O
    name, vtx, xyz, nparts = make_mesh(kind)
    threads = O.threads(0)
    lv = O.RsbLevels(vtx, xyz, nparts)
    levels = []
    t_all = time.time()
    for L in range(lv.ncuts):
        it0, rows0 = lv.info.total_iters, lv.info.row_iters
        t0 = time.time()
        lv.level()
        levels.append({"level": L, "groups": int(len(lv.segs) // 2),
                       "lanczos_steps": int(lv.info.total_iters - it0),
                       "row_steps": int(lv.info.row_iters - rows0),
                       "wall_s_here": round(time.time() - t0, 2)})
        print(name, levels[-1], flush=True)
    part = lv.part()
    q = O.part_quality(part, vtx, nparts)
    out = {
        "workload": name, "nparts": nparts, "elements": int(len(vtx)),
        "mesh_sha256": {"vtx": sha(vtx), "xyz": sha(xyz)},
        "options": {"rsb_algo": 0, "rsb_pre": 1, "rsb_tol": 1e-5, "rsb_max_iter": 50,
                    "rsb_max_passes": 50},
        "weighted_cut": q[0], "cut_pairs": q[1], "imbalance": q[5], "comm_volume": q[6],
        "part_sizes": np.bincount(part, minlength=nparts).tolist(),
        "part_sha256": sha(part.astype(np.int32)),
        "lanczos_steps": int(lv.info.total_iters), "row_steps": int(lv.info.row_iters),
        "unconverged": int(lv.info.unconverged), "max_components": int(lv.info.max_components),
        "max_fiedler_resid": lv.info.max_resid, "levels": levels,
        "oracle_threads_here": threads, "wall_s_here": round(time.time() - t_all, 1),
    }
    path = os.path.join(HERE, f"rsb_{name}.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", path, "cut", q[0])


if __name__ == "__main__":
    which = sys.argv[1] if len(sys.argv) > 1 else "all"
    for k in (["pipe", "box"] if which == "all" else [which]):
        run(k)
