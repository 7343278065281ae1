"""Generates the golden fixtures of tests/test_golden.py (run from the repo
root: ``python tests/golden/make_golden.py``).

The reference cannot be built here (a Rust crate; no toolchain), so the
fixtures hold the faithful f64 oracle's answers (the reference's algorithm in
its own operation order, `oracle/rayna_oracle.hpp` RefF64) on seeded ray
suites, and the colours a ray sees through textures and the image sky. They
pin the oracle in history: a change to the oracle, the flattener or the
seeded scenes that moves an answer shows up as a fixture mismatch, and the
device is held to the same fixtures on the GPU.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from oracle import binding as ob  # noqa: E402
from rayna_gb300 import presets  # noqa: E402
from rayna_gb300.scene import Scene, flatten  # noqa: E402

import raysuite as rs  # noqa: E402

N_RAYS = 1000


def suites():
    """(name, scene, origins, directions) of every fixture suite, seeded."""
    out = []
    rng = np.random.Generator(np.random.PCG64(101))
    out.append(("spheres", rs.sphere_scene(), *rs.rays_at(rng, N_RAYS, (-12, -1, -12), (12, 2.5, 12))))
    rng = np.random.Generator(np.random.PCG64(102))
    scene, verts = rs.triangle_scene(level=3)
    out.append(("triangles", scene, *rs.rays_at(rng, N_RAYS, (0, 0, 0), (1, 1, 1), targets=verts.reshape(-1, 3))))
    rng = np.random.Generator(np.random.PCG64(103))
    out.append(("boxes", rs.box_scene(), *rs.rays_at(rng, N_RAYS, (-3.5, -3.5, -3.5), (3.5, 3.5, 3.5))))
    rng = np.random.Generator(np.random.PCG64(104))
    out.append(("planar", rs.planar_scene(), *rs.rays_at(rng, N_RAYS, (-3, -3, -3), (3, 3, 3))))
    rng = np.random.Generator(np.random.PCG64(105))
    out.append(("transformed", rs.transform_scene(seed=5), *rs.rays_at(rng, N_RAYS, (-3.5, -3.5, -3.5), (3.5, 3.5, 3.5))))
    rng = np.random.Generator(np.random.PCG64(106))
    out.append(("cornell", presets.cornell()[0], *rs.rays_at(rng, N_RAYS, (0.02, 0.02, 0.02), (0.98, 0.98, 0.98))))
    rng = np.random.Generator(np.random.PCG64(107))
    s = rs.sdf_scene()
    out.append(("sdf_analytic", Scene(objects=[s.objects[0], s.objects[1], s.objects[3]]),
                *rs.rays_at(rng, N_RAYS // 2, (-1.5, -1, -1.5), (3.2, 2, 1.5))))
    return out


def colour_suite():
    """The textured demo scene: rays from the camera region into the scene
    and the sky, for the colour each one sees."""
    scene, cam, _ = presets.textures_demo()
    rng = np.random.Generator(np.random.PCG64(108))
    o = np.tile(np.array([0.0, 2.2, 8.0]), (N_RAYS, 1)) + rng.normal(scale=0.3, size=(N_RAYS, 3))
    tgt = rng.uniform((-4, -0.5, -3), (4, 4, 3), (N_RAYS, 3))
    return scene, o.astype(np.float32), (tgt - o).astype(np.float32)


def main():
    arrays = {}
    for name, scene, o, d in suites():
        flat = flatten(scene)
        h, t64, n64 = ob.query(flat, o, d, policy=ob.POLICY_REF_F64, pretest=True)
        arrays[f"{name}_o"] = o
        arrays[f"{name}_d"] = d
        arrays[f"{name}_hit"] = h["hit"].astype(np.uint8)
        arrays[f"{name}_prim"] = h["prim"].astype(np.uint32)
        arrays[f"{name}_t"] = t64
        arrays[f"{name}_n"] = n64
        print(f"{name}: {int(h['hit'].sum())} hits of {len(o)}")
    scene, o, d = colour_suite()
    arrays["colour_o"], arrays["colour_d"] = o, d
    arrays["colour_rgb"] = ob.query_colour(flatten(scene), o, d, ob.POLICY_REF_F64)
    path = os.path.join(HERE, "oracle_f64.npz")
    np.savez_compressed(path, **arrays)
    print(path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
