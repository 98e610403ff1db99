"""Golden outputs of the reference's own compute shaders, run on the CPU
through oracle/ref_shaders.cpp (PathTracer.comp and ShadowVolume.comp,
transliterated by oracle/build_ref.py), for tests/test_ref_shader_golden.py,
which checks the oracle against them on machines without the reference tree.

    python tests/golden/make_ref_shader_golden.py   # needs the reference tree

Writes tests/golden/ref_shaders.npz.  `scenes()` is the single definition of
the inputs, shared with the test.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, "cloudrendering-vulkan_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

OUT = os.path.join(HERE, "ref_shaders.npz")


def scenes():
    """The inputs: two clouds with camera, reference-parity parameters and
    shadow volume, plus the RNG seeds and scattering inputs."""
    import vcr
    from vcr import configs
    from oracle import oracle as orc

    out = {}
    for name, size, ds, g, W, H, seed, sv_n in (("a", (32, 32, 32), 6.0, 0.857, 48, 48, 12345, 24),
                                                ("b", (48, 40, 48), 16.0, 0.0, 40, 30, 777, 24)):
        dense = orc.fbm_fill(size, seed=3, octaves=5)
        og = orc.Grid(dense, 0)
        cloud = vcr.cloud_from_grid(vcr.grid_desc(size, (1 / max(size),) * 3), 1.0, ds)
        cloud.max_extinction = max(og.max_density(), 0.01)
        sv = vcr.shadow_volume_setup(configs.sun_travel_dir(), cloud.bounds_min, cloud.bounds_max, sv_n)
        cam = vcr.camera_look((0.0, 0.0, -0.6), (0.0, 0.0, 1.0), 70.0, 0.1, W, H)
        p = configs.C1_PT.params(vcr.TRACKER_GLOBAL)
        vcr.params_set_phase_g(p, g)
        p.albedo, p.max_events = 1.0, 0
        p.rng_mode, p.nee_mode, p.sky_mode = vcr.RNG_XORSHIFT, vcr.NEE_SHADOW_VOLUME, vcr.SKY_GRADIENT
        out[name] = dict(dense=dense, og=og, cloud=cloud, sv=sv, cam=cam, params=p, W=W, H=H, seed=seed)
    rng = np.random.default_rng(5)
    d = rng.normal(size=(200, 3))
    out["seeds"] = rng.integers(0, 2 ** 32, 100, dtype=np.uint64).astype(np.uint32)
    out["scatter_in"] = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    out["scatter_state"] = rng.integers(1, 2 ** 32, 200, dtype=np.uint64).astype(np.uint32)
    return out


def main():
    from oracle import ref_shaders as rs
    from oracle.oracle import _p

    s = scenes()
    L = rs.lib()
    res = {}
    for name in ("a", "b"):
        c = s[name]
        sv_ref = rs.sv_build(rs.Scene(c["dense"], c["cloud"], c["cam"], c["params"], c["sv"], None))
        # the path tracer reads the reference's own shadow volume
        img = rs.pt_image(rs.Scene(c["dense"], c["cloud"], c["cam"], c["params"], c["sv"], sv_ref), c["W"], c["H"],
                          c["seed"])
        res[f"sv_{name}"] = sv_ref
        res[f"pt_{name}"] = img[..., :3].copy()
    res["init_states"] = np.array([L.ref_initialize_random(int(v)) for v in s["seeds"]], np.uint32)
    nums = np.zeros(1000, np.float32)
    res["numbers_state_after"] = np.array([L.ref_random_numbers(12345, 1000, _p(nums))], np.uint32)
    res["numbers"] = nums
    outs, states = np.zeros((200, 3), np.float32), np.zeros(200, np.uint32)
    rs.Scene(s["a"]["dense"], s["a"]["cloud"], s["a"]["cam"], s["a"]["params"], s["a"]["sv"], None)  # g = 0.857
    for i, (d, st) in enumerate(zip(s["scatter_in"], s["scatter_state"])):
        o = np.zeros(3, np.float32)
        states[i] = L.ref_scatter_ray(_p(np.ascontiguousarray(d)), int(st), _p(o))
        outs[i] = o
    res["scatter_out"], res["scatter_state_after"] = outs, states
    np.savez_compressed(OUT, **res)
    print(f"wrote {OUT} ({os.path.getsize(OUT)} bytes)")


if __name__ == "__main__":
    main()
