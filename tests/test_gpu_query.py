"""Ray-query parity on the GPU, through the C ABI (rg_query_rays).

For closed-form primitives (sphere, triangle, box, torus and sphere SDFs) the
arithmetic-contract build must be bit-exact against the f32 oracle that
follows the kernels' operation order, evaluated by brute force over every
primitive (no bounding volumes): same hit/miss, same primitive (up to
exact-distance ties), same distance and normal bits. The device's slab test
is conservative, so its BVH never changes which primitive is closest.

Against the faithful f64 oracle, on every suite and in both builds (the
performance build fuses multiply-adds where the compiler finds them):

* hit/miss agrees on at least 99.9% of rays (99.8% on the planar suite);
* where the two pick different primitives, the disagreements are counted,
  bounded per suite, and must be near-ties: the f32 distance still within
  tolerance of the f64 closest distance;
* the distance agrees within 1e-5 relative, or within the first-order f32
  error bound of the primitive's formula where that bound is larger
  (ill-conditioned hits: counted and reported);
* the outward normal agrees within 1e-5 (normals are unit vectors, so
  absolute = relative), or within the first-order f32 error bound of the
  normal's formula (the f32 distance error divided by the radius for
  spheres, the barycentric error times the vertex-normal spread for
  triangles, the central difference's rounding divided by its step for
  raymarched surfaces); the fraction beyond 1e-5 is reported.

Media (free-flight logarithm) and the Mandelbulb (transcendental distance
estimator) use library transcendentals on both sides and are held to
tolerances stated in each test.
"""
import numpy as np
import pytest

from oracle import binding as ob
from rayna_gb300 import Renderer, presets
from rayna_gb300.scene import Camera, RenderOpts, flatten

from raysuite import (
    box_scene, planar_scene, rays_at, sdf_scene, sphere_scene, transform_scene, triangle_scene, volume_scene,
)

pytestmark = pytest.mark.gpu
EPS32 = np.finfo(np.float32).eps


def renderer_for(scene, bvh_width=2, exact=True):
    r = Renderer.new_from(scene, Camera(), RenderOpts(width=8, height=8), exact=exact)
    r.set_tuning(bvh_width=bvh_width)
    assert r.tuning()["bvh_width"] == bvh_width
    return r


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def compare_bit_exact(g, h, label):
    assert np.array_equal(g["hit"], h["hit"]), f"{label}: hit/miss differs on {np.sum(g['hit'] != h['hit'])} rays"
    m = g["hit"] == 1
    assert np.array_equal(bits(g["t"][m]), bits(h["t"][m])), f"{label}: distance bits differ"
    prim_diff = m & (g["prim"] != h["prim"])
    # a different primitive is allowed only at an exact-distance tie (same t bits)
    assert np.all(bits(g["t"][prim_diff]) == bits(h["t"][prim_diff]))
    same = m & (g["prim"] == h["prim"])
    assert np.array_equal(bits(g["normal"][same]), bits(h["normal"][same])), f"{label}: normal bits differ"
    assert np.array_equal(bits(g["ray_normal"][same]), bits(h["ray_normal"][same])), f"{label}: ray_normal bits differ"
    assert np.array_equal(g["front_face"][same], h["front_face"][same])
    assert np.array_equal(g["material"][same], h["material"][same])
    return int(m.sum()), int(prim_diff.sum())


def f64_error_bound(flat, o, d, prim, t64):
    """First-order f32 error bound of the distance for each hit."""
    o = o.astype(np.float64)
    d = d.astype(np.float64) / np.linalg.norm(d, axis=1, keepdims=True)
    ns, nt = flat.desc.n_spheres, flat.desc.n_triangles
    bound = 8 * EPS32 * (np.abs(o).max(axis=1) + t64)
    s = prim < ns
    if s.any():
        sp = flat.a_spheres[prim[s]].astype(np.float64)
        oc = o[s] - sp[:, :3]
        hb = np.einsum("ij,ij->i", oc, d[s])
        cc = np.einsum("ij,ij->i", oc, oc) - sp[:, 3] ** 2
        sq = np.sqrt(np.maximum(hb * hb - cc, 1e-300))
        occ = np.einsum("ij,ij->i", oc, oc) + sp[:, 3] ** 2
        bound[s] += 4 * EPS32 * (occ / (2 * sq) + np.abs(hb) + np.linalg.norm(oc, axis=1) + np.abs(sp[:, :3]).max(axis=1))
    tr = (prim >= ns) & (prim < ns + nt)
    if tr.any():
        v = flat.a_tri_v[prim[tr] - ns].astype(np.float64)
        e1, e2 = v[:, 1] - v[:, 0], v[:, 2] - v[:, 0]
        det = np.abs(np.einsum("ij,ij->i", e1, np.cross(d[tr], e2)))
        amp = np.linalg.norm(e1, axis=1) * np.linalg.norm(e2, axis=1) / np.maximum(det, 1e-300)
        bound[tr] += 16 * EPS32 * amp * (t64[tr] + np.linalg.norm(o[tr] - v[:, 0], axis=1))
    D = flat.desc
    q0 = ns + nt + D.n_boxes + D.n_volumes + D.n_sdfs
    c0 = q0 + D.n_quads
    p0 = c0 + D.n_cylinders

    def planar_bound(sel, rows):
        # t = -(n.o + d) / (n.dir): relative error of the numerator, amplified by 1 / |n.dir|
        pts = rows[:, 0:3].astype(np.float64)
        n = np.cross(rows[:, 3:6], rows[:, 6:9]).astype(np.float64)
        n /= np.linalg.norm(n, axis=1, keepdims=True)
        # rounding of the numerator, and of the denominator (relative to sum |n_i dir_i|) times t
        den = np.abs(np.einsum("ij,ij->i", n, d[sel]))
        sabs = np.einsum("ij,ij->i", np.abs(n), np.abs(d[sel]))
        num = np.abs(o[sel]).sum(axis=1) + np.abs(pts).sum(axis=1) + t64[sel] * sabs
        return 16 * EPS32 * num / np.maximum(den, 1e-300)

    qs = (prim >= q0) & (prim < c0)
    if qs.any():
        bound[qs] += planar_bound(qs, flat.a_quads[prim[qs] - q0])
    ps = prim >= p0
    if ps.any():
        bound[ps] += planar_bound(ps, flat.a_planes[prim[ps] - p0])
    cs = (prim >= c0) & (prim < p0)
    if cs.any():
        # the cylinder quadratic a t^2 + 2 b t + c with a, b, c scaled by |p2 - p1|^2: rounding of b and of the
        # discriminant, divided by a (small for rays near the axis direction)
        cy = flat.a_cyls[prim[cs] - c0].astype(np.float64)
        al = cy[:, 3:6] - cy[:, 0:3]
        l2 = np.einsum("ij,ij->i", al, al)
        oc = o[cs] - cy[:, 0:3]
        bard = np.einsum("ij,ij->i", al, d[cs])
        baoc = np.einsum("ij,ij->i", al, oc)
        a = l2 - bard * bard
        b = l2 * np.einsum("ij,ij->i", oc, d[cs]) - baoc * bard
        c = l2 * np.einsum("ij,ij->i", oc, oc) - baoc * baoc - cy[:, 6] ** 2 * l2
        disc = np.maximum(b * b - c * a, 1e-300)
        scale = l2 * (np.einsum("ij,ij->i", oc, oc) + cy[:, 6] ** 2 + 1.0)
        db = 8 * EPS32 * scale
        dsq = 8 * EPS32 * (b * b + np.abs(c * a) + scale * scale) / (2 * np.sqrt(disc))
        bound[cs] += (db + dsq) / np.maximum(np.abs(a), 1e-300) + 8 * EPS32 * (l2 + np.abs(baoc)) / np.maximum(np.abs(bard), 1e-300)
    return bound


def normal_error_bound(flat, o, d, prim, t64, dt):
    """First-order f32 error bound of the outward normal of each hit (on top
    of a few ulps of the normalisation)."""
    o = o.astype(np.float64)
    d = d.astype(np.float64) / np.linalg.norm(d, axis=1, keepdims=True)
    ns, nt = flat.desc.n_spheres, flat.desc.n_triangles
    bound = np.full(len(prim), 8 * EPS32)
    s = prim < ns
    if s.any():  # (p - c) / r with p = o + t d
        sp = flat.a_spheres[prim[s]].astype(np.float64)
        scale = np.abs(o[s]).max(axis=1) + t64[s] + np.abs(sp[:, :3]).max(axis=1) + sp[:, 3]
        bound[s] += (np.abs(dt[s]) + 8 * EPS32 * scale) / sp[:, 3]
    tr = (prim >= ns) & (prim < ns + nt)
    if tr.any():  # sum_i b_i n_i with the barycentric errors of Moller-Trumbore
        v = flat.a_tri_v[prim[tr] - ns].astype(np.float64)
        n = flat.a_tri_n[prim[tr] - ns].astype(np.float64)
        e1, e2 = v[:, 1] - v[:, 0], v[:, 2] - v[:, 0]
        det = np.maximum(np.abs(np.einsum("ij,ij->i", e1, np.cross(d[tr], e2))), 1e-300)
        dist = np.linalg.norm(o[tr] - v[:, 0], axis=1) + t64[tr]
        du = 16 * EPS32 * dist * np.linalg.norm(e2, axis=1) / det
        dv = 16 * EPS32 * dist * np.linalg.norm(e1, axis=1) / det
        bound[tr] += du * np.linalg.norm(n[:, 1] - n[:, 0], axis=1) + dv * np.linalg.norm(n[:, 2] - n[:, 0], axis=1)
    D = flat.desc
    c0 = ns + nt + D.n_boxes + D.n_volumes + D.n_sdfs + D.n_quads
    cy = (prim >= c0) & (prim < c0 + D.n_cylinders)
    if cy.any():  # body normal (p - p1 - axis * along) / radius, p = o + t d
        cyl = flat.a_cyls[prim[cy] - c0].astype(np.float64)
        scale = np.abs(o[cy]).max(axis=1) + t64[cy] + np.abs(cyl[:, :6]).max(axis=1)
        bound[cy] += 2 * (np.abs(dt[cy]) + 8 * EPS32 * scale) / cyl[:, 6]
    s0 = ns + nt + D.n_boxes + D.n_volumes
    sd = (prim >= s0) & (prim < s0 + D.n_sdfs)
    if sd.any():  # central differences of the SDF with step eps: rounding of each evaluation / (2 eps)
        for k in np.unique(prim[sd] - s0):
            f = flat.c_sdfs[int(k)]
            sel = sd & (prim - s0 == k)
            p = o[sel] + d[sel] * t64[sel, None]
            mag = np.abs(p).max(axis=1) + max(abs(f.centre[0]), abs(f.centre[1]), abs(f.centre[2])) + abs(f.params[0])
            bound[sel] += 16 * EPS32 * mag / f.epsilon + np.abs(dt[sel]) / max(f.params[1], f.params[0], 1e-3)
    return bound


def sdf_distance_bound(flat, prim, d, n64):
    """Sphere tracing stops within epsilon of the surface in either
    precision: the distance can differ by about epsilon over the cosine of
    the incidence."""
    D = flat.desc
    s0 = flat.desc.n_spheres + flat.desc.n_triangles + D.n_boxes + D.n_volumes
    out = np.zeros(len(prim))
    sd = (prim >= s0) & (prim < s0 + D.n_sdfs)
    if sd.any():
        dn = d[sd].astype(np.float64) / np.linalg.norm(d[sd], axis=1, keepdims=True)
        cos = np.abs(np.einsum("ij,ij->i", dn, n64[sd]))
        eps = np.array([flat.c_sdfs[int(k)].epsilon for k in prim[sd] - s0])
        out[sd] = 4 * eps / np.maximum(cos, 0.05)
    return out


def compare_f64(flat, o, d, g, label, min_agree=0.999, max_prim_diff=0.002, max_leak=0.0):
    """Device hits g against the faithful f64 oracle; returns a dict of the
    agreement figures (asserting the bars in the module docstring)."""
    h, t64, n64 = ob.query(flat, o, d, policy=ob.POLICY_REF_F64, pretest=True)
    agree = np.mean(g["hit"] == h["hit"])
    assert agree >= min_agree, f"{label}: hit agreement with f64 {agree:.5f}"
    both = (g["hit"] == 1) & (h["hit"] == 1)
    t32 = g["t"].astype(np.float64)
    bnd_t = np.zeros(len(o))
    bnd_t[both] = f64_error_bound(flat, o[both], d[both], g["prim"][both], t64[both])
    bnd_t[both] += sdf_distance_bound(flat, g["prim"][both], d[both], n64[both])
    rel = np.abs(t32 - t64) / np.maximum(np.abs(t64), 1e-30)
    t_ok = (rel <= 1e-5) | (np.abs(t32 - t64) <= bnd_t)
    # a different primitive: counted, and only at a near-tie of distance, or
    # where the reference's cylinder rule (order-dependent, the f64 oracle
    # keeps it) returns a farther hit than the closest one the device reports
    pdiff = both & (g["prim"] != h["prim"])
    frac_pdiff = pdiff.sum() / max(both.sum(), 1)
    assert frac_pdiff <= max_prim_diff, f"{label}: {pdiff.sum()} primitive disagreements ({frac_pdiff:.5f})"
    D = flat.desc
    c0 = D.n_spheres + D.n_triangles + D.n_boxes + D.n_volumes + D.n_sdfs + D.n_quads
    is_cyl = lambda pr: (pr >= c0) & (pr < c0 + D.n_cylinders)
    cyl_rule = pdiff & (is_cyl(g["prim"]) | is_cyl(h["prim"])) & (t32 < t64)
    # Moller-Trumbore is not watertight (triangle.rs:53-109 rejects u, v
    # outside [0, 1] with rounding either side of a shared edge): a ray aimed
    # exactly at a shared vertex can pass between the triangles in one
    # precision and hit one of them in the other, then hit something behind
    leak = pdiff & ~t_ok & ~cyl_rule
    frac_leak = leak.sum() / max(both.sum(), 1)
    assert frac_leak <= max_leak, f"{label}: {leak.sum()} primitive disagreements that are not near-ties ({frac_leak:.5f})"
    m = both & ~pdiff
    assert t_ok[m].all(), f"{label}: {np.sum(~t_ok[m])} distances outside tolerance; worst rel {rel[m][~t_ok[m]].max()}"
    ill = float(np.mean(rel[m] > 1e-5)) if m.any() else 0.0
    # outward normals
    n32 = g["normal"].astype(np.float64)
    nerr = np.abs(n32 - n64).max(axis=1)
    nb = np.zeros(len(o))
    nb[m] = normal_error_bound(flat, o[m], d[m], g["prim"][m], t64[m], (t32 - t64)[m])
    n_ok = (nerr <= 1e-5) | (nerr <= nb)
    assert n_ok[m].all(), (f"{label}: {np.sum(~n_ok[m])} normals outside tolerance; worst {nerr[m][~n_ok[m]].max():.3e}"
                           f" (bound {nb[m][~n_ok[m]].max():.3e})")
    n_beyond = float(np.mean(nerr[m] > 1e-5)) if m.any() else 0.0
    return {"agree": float(agree), "prim_diff": float(frac_pdiff), "cylinder_rule": int(cyl_rule.sum()),
            "edge_leaks": int(leak.sum()), "t_ill": ill,
            "t_median_rel": float(np.median(rel[m])) if m.any() else 0.0, "normal_beyond_1e-5": n_beyond,
            "normal_median": float(np.median(nerr[m])) if m.any() else 0.0, "hits": int(m.sum())}


def axis_aligned_rays(rng, n, lo, hi):
    """Rays whose directions have exact zero components (along an axis or in
    an axis plane): the traversal's zero-direction handling."""
    lo, hi = np.asarray(lo, np.float32), np.asarray(hi, np.float32)
    o = rng.uniform(lo, hi, (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    zero = rng.integers(0, 3, n)
    d[np.arange(n), zero] = 0.0
    both = rng.random(n) < 0.5
    d[np.arange(n)[both], (zero[both] + 1) % 3] = 0.0
    return o, d


SUITES = ["spheres", "triangles", "mesh", "boxes", "sdf_analytic", "axis_aligned", "planar", "transformed",
          "transformed_scaled", "cornell"]


def suite_rays(suite):
    seeds = {"spheres": 1, "triangles": 2, "mesh": 7, "boxes": 3, "sdf_analytic": 4, "axis_aligned": 8, "planar": 9,
             "transformed": 10, "transformed_scaled": 11, "cornell": 12}
    rng = np.random.Generator(np.random.PCG64(seeds[suite]))
    if suite == "spheres":
        scene = sphere_scene()
        o, d = rays_at(rng, 20000, (-12, -1, -12), (12, 2.5, 12))
    elif suite == "triangles":
        scene, verts = triangle_scene(level=4)
        o, d = rays_at(rng, 20000, (0, 0, 0), (1, 1, 1), targets=verts.reshape(-1, 3))
    elif suite == "mesh":
        scene = presets.cornell_mesh(level=5)[0]
        o, d = rays_at(rng, 10000, (0.02, 0.02, 0.02), (0.98, 0.98, 0.98))
    elif suite == "planar":
        scene = planar_scene()
        o, d = rays_at(rng, 20000, (-3, -3, -3), (3, 3, 3))
    elif suite in ("transformed", "transformed_scaled"):
        scene = transform_scene(seed=5, rigid=suite == "transformed")
        o, d = rays_at(rng, 20000, (-3.5, -3.5, -3.5), (3.5, 3.5, 3.5))
    elif suite == "cornell":
        scene = presets.cornell()[0]
        o, d = rays_at(rng, 10000, (0.02, 0.02, 0.02), (0.98, 0.98, 0.98))
    elif suite == "axis_aligned":
        scene = presets.cornell_mesh(level=4)[0]
        o, d = axis_aligned_rays(rng, 10000, (0.02, 0.02, 0.02), (0.98, 0.98, 0.98))
    elif suite == "boxes":
        scene = box_scene()
        o, d = rays_at(rng, 20000, (-3.5, -3.5, -3.5), (3.5, 3.5, 3.5))
    else:
        from rayna_gb300.scene import Scene
        s = sdf_scene()
        scene = Scene(objects=[s.objects[0], s.objects[1], s.objects[3]])
        o, d = rays_at(rng, 4000, (-1.5, -1, -1.5), (3.2, 2, 1.5))
    return scene, o, d


@pytest.mark.parametrize("bvh_width", [2, 8])
@pytest.mark.parametrize("suite", SUITES)
def test_query_bit_exact_vs_f32_oracle(suite, bvh_width):
    scene, o, d = suite_rays(suite)
    flat = flatten(scene)
    with renderer_for(scene, bvh_width) as r:
        g = r.query_rays(o, d)
    h, _, _ = ob.query(flat, o, d, policy=ob.POLICY_GPU_F32, pretest="brute")
    nhit, nties = compare_bit_exact(g, h, suite)
    assert nhit > 0.2 * len(o)
    print(f"{suite} (bvh width {bvh_width}): {nhit} hits bit-exact, {nties} exact-distance ties")


# Suites compared with the faithful f64 oracle. transformed_scaled is left
# out on purpose: under scaling the reference bounds a mesh-space distance by
# the world-space interval end, so its closest hit depends on the order of
# its traversal (about one ray in six on this suite); the device returns the
# closest world-space hit, which the rigid `transformed` suite and the f32
# oracle pin instead.
F64_SUITES = [s for s in SUITES if s != "transformed_scaled"]
# Primitive disagreements allowed per suite (fraction of hits both sides
# report): shared edges and vertices of meshes, coplanar box faces, and the
# reference's order-dependent cylinder rule give near-ties whose winner f32
# rounding decides.
MAX_PRIM_DIFF = {"planar": 0.004, "mesh": 0.004, "axis_aligned": 0.004,
                 # rays aimed at the mesh's vertices: every hit is on edges shared by up to six triangles
                 "triangles": 0.08,
                 # rays along the walls of the rotated boxes and the box edges
                 "cornell": 0.025}


@pytest.mark.parametrize("exact", [True, False])
@pytest.mark.parametrize("suite", F64_SUITES)
def test_query_vs_f64_oracle(suite, exact):
    scene, o, d = suite_rays(suite)
    flat = flatten(scene)
    with renderer_for(scene, 2, exact=exact) as r:
        g = r.query_rays(o, d)
    st = compare_f64(flat, o, d, g, suite, min_agree=0.998 if suite == "planar" else 0.999,
                     max_prim_diff=MAX_PRIM_DIFF.get(suite, 0.002), max_leak=0.03 if suite == "triangles" else 0.0)
    build = "exact" if exact else "performance"
    print(f"{suite} ({build} build) vs f64: {st}")


@pytest.mark.parametrize("level", [8])
def test_query_full_mesh_vs_oracles(level):
    """The benchmarked triangle-mesh workload itself (1,310,732 triangles):
    bit-exact against the f32 oracle's BVH walk and within the f64 bars."""
    scene = presets.cornell_mesh(level=level)[0]
    flat = flatten(scene)
    rng = np.random.Generator(np.random.PCG64(80 + level))
    o, d = rays_at(rng, 20000, (0.02, 0.02, 0.02), (0.98, 0.98, 0.98))
    # half of the rays aimed at the displaced sphere's surface
    c = np.array([0.5, 0.3, 0.5])
    dirs = rng.normal(size=(10000, 3))
    tgt = c + 0.25 * dirs / np.linalg.norm(dirs, axis=1, keepdims=True)
    d[:10000] = (tgt - o[:10000]).astype(np.float32)
    with renderer_for(scene, 2) as r:
        g = r.query_rays(o, d)
    with renderer_for(scene, 8) as r:
        g8 = r.query_rays(o, d)
    h, _, _ = ob.query(flat, o, d, policy=ob.POLICY_GPU_F32, pretest=False)
    nhit, nties = compare_bit_exact(g, h, "mesh level 8")
    compare_bit_exact(g8, h, "mesh level 8, 8-wide")
    st = compare_f64(flat, o, d, g, "mesh level 8", max_prim_diff=0.004)
    print(f"mesh level {level}: {nhit} hits bit-exact, {nties} ties; vs f64: {st}")


@pytest.mark.parametrize("bvh_width", [2, 8])
@pytest.mark.parametrize("transformed", [False, True])
def test_query_volumes_injected_uniforms(bvh_width, transformed):
    rng = np.random.Generator(np.random.PCG64(5))
    scene = volume_scene(transformed)
    flat = flatten(scene)
    o, d = rays_at(rng, 20000, (-1.2, -1.2, -1.2), (2.7, 1.2, 1.2), inside_frac=0.3)
    u = rng.uniform(1e-6, 1.0, (len(o), flat.desc.n_volumes)).astype(np.float32)
    with renderer_for(scene, bvh_width) as r:
        g = r.query_rays(o, d, volume_u=u)
    h, _, _ = ob.query(flat, o, d, volume_u=u, policy=ob.POLICY_GPU_F32, pretest=False)
    agree = np.mean((g["hit"] == h["hit"]) & ((g["hit"] == 0) | (g["prim"] == h["prim"])))
    assert agree >= 0.9995, agree
    m = (g["hit"] == 1) & (h["hit"] == 1) & (g["prim"] == h["prim"])
    rel = np.abs(g["t"][m].astype(np.float64) - h["t"][m]) / np.maximum(np.abs(h["t"][m]), 1e-30)
    assert rel.max() <= 2e-6, rel.max()   # logf on both sides: a few ulps
    vol = m & (g["prim"] >= flat.desc.n_spheres)
    assert vol.sum() > 1000
    hf, t64, _ = ob.query(flat, o, d, volume_u=u, policy=ob.POLICY_REF_F64, pretest=True)
    agree64 = np.mean(g["hit"] == hf["hit"])
    assert agree64 >= 0.999, agree64


@pytest.mark.parametrize("exact", [True, False])
def test_query_mandelbulb_tolerance(exact):
    rng = np.random.Generator(np.random.PCG64(6))
    from rayna_gb300.scene import Scene
    s = sdf_scene()
    scene = Scene(objects=[s.objects[2]])
    flat = flatten(scene)
    o, d = rays_at(rng, 3000, (-3.7, -1.2, -1.2), (-1.3, 1.2, 1.2), inside_frac=0.0)
    with renderer_for(scene, exact=exact) as r:
        g = r.query_rays(o, d)
    h, _, _ = ob.query(flat, o, d, policy=ob.POLICY_GPU_F32, pretest=False)
    agree = np.mean(g["hit"] == h["hit"])
    assert agree >= 0.99, agree
    m = (g["hit"] == 1) & (h["hit"] == 1)
    assert m.sum() > 300
    err = np.abs(g["t"][m] - h["t"][m])
    assert np.mean(err <= 1e-3) >= 0.99, np.quantile(err, 0.99)
    # the distance estimator is the same sequence of IEEE operations on both
    # sides (its logarithm included), so the marches agree bit for bit
    same = np.mean(bits(g["t"][m]) == bits(h["t"][m]))
    print(f"mandelbulb: {same:.5f} of hits bit-exact")
    assert same >= 0.999, same
