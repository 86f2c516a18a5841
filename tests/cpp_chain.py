"""Builds and drives tests/cpp/ops_chain.cpp, the C++ operator chain over
include/trax_ops.hpp."""
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "ops_chain.cpp")
LIBDIR = os.path.join(ROOT, "trax_gb300")

OUTPUTS = ("grid", "orig", "pairs", "pair_offsets", "cands", "cand_offsets", "hit1", "hit2",
           "hit3", "trk_offsets", "connectivity")


def compile_chain(out_dir):
    exe = os.path.join(out_dir, "ops_chain")
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror",
                    "-I" + os.path.join(ROOT, "include"), SRC, "-L" + LIBDIR, "-ltrax_gb300",
                    "-Wl,-rpath," + LIBDIR, "-o", exe], check=True)
    return exe


def write_input(path, b, cfg, grid):
    with open(path, "wb") as f:
        hdr = np.array([b.n_hits, b.n_events, b.n_layers, grid.n_sectors_z, grid.n_sectors_phi,
                        cfg.n_layer_triplets, cfg.n_geom_layers], np.uint32)
        f.write(hdr.tobytes())
        f.write(np.float32(cfg.min_pt).tobytes())
        for a in (b.x, b.y, b.z):
            f.write(np.ascontiguousarray(a, np.float32).tobytes())
        for a in (b.layer, b.detector_id, b.hit_id, b.event, b.layer_nhits):
            f.write(np.ascontiguousarray(a, np.uint32).tobytes())
        for i in range(cfg.n_layer_triplets):
            f.write(bytes(cfg.triplets[i]))
        ng = cfg.n_geom_layers
        f.write(np.array(cfg.min_radius[:ng], np.float32).tobytes())
        f.write(np.array(cfg.max_radius[:ng], np.float32).tobytes())


def read_output(path):
    raw = np.fromfile(path, np.uint32)
    out, pos = {}, 0
    for name in OUTPUTS:
        n = int(raw[pos])
        out[name] = raw[pos + 1:pos + 1 + n]
        pos += 1 + n
    assert pos == raw.size
    out["pairs"] = out["pairs"].reshape(-1, 2)
    out["cands"] = out["cands"].reshape(-1, 2)
    return out


def run_chain(exe, b, cfg, grid, work_dir, pair_generator="beamspot"):
    inp, outp = os.path.join(work_dir, "in.bin"), os.path.join(work_dir, "out.bin")
    write_input(inp, b, cfg, grid)
    p = subprocess.run([exe, inp, outp, pair_generator], capture_output=True, text=True)
    return p, (read_output(outp) if p.returncode == 0 else None)
