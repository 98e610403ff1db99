"""Standalone grid tool: the .xyz format (Grid3D.h: Load :44-90, Save
:166-178; GridData.h:14-25), the seeded fBm generator that stands in for the
reference's cloud file, and the bricking the trackers render from.

    python -m vcr.grid_tool generate --size 256 256 256 --seed 1 --octaves 6 -o cloud.xyz [--device]
    python -m vcr.grid_tool info cloud.xyz
    python -m vcr.grid_tool convert cloud.xyz --precision fp16 -o cloud_fp16.xyz
    python -m vcr.grid_tool slice cloud.xyz --axis z --index 128 -o slice.png

`generate` runs the generator on the host, or with --device on the GPU and
reads the grid back; `convert` stores the grid as bricks of the given
precision on the GPU and writes what the trackers sample (FP16 / BF16 texels
times their brick's scale) back to a .xyz file, with the error it made;
`info` prints the header, GetMajorant (Grid3D.h:180-192) and what the grid
takes on the device per precision.
"""
from __future__ import annotations

import argparse
import json
import sys

import numpy as np

from . import _abi
from . import Context, fbm_desc, fbm_fill_host, grid_desc, write_png, xyz_read, xyz_write

PRECISIONS = {"fp32": _abi.PREC_FP32, "fp16": _abi.PREC_FP16, "bf16": _abi.PREC_BF16}


def device_bytes(size, precision: str) -> dict:
    """Bytes the stored grid takes: bricks of 8^3 texels, one FP32 scale per
    brick, majorant pyramid levels 0..3 (one float per cell, each level
    padded to 16 bytes)."""
    nb = [(n + 7) // 8 for n in size]
    bricks = nb[0] * nb[1] * nb[2]
    texel = 4 if precision == "fp32" else 2
    pyramid, m = 0, list(nb)
    for _ in range(4):
        pyramid += ((m[0] * m[1] * m[2] + 3) // 4) * 16
        m = [(v + 1) // 2 for v in m]
    scales = bricks * 4
    return {"bricks": bricks * 512 * texel, "scales": scales, "majorants": pyramid,
            "total": bricks * 512 * texel + scales + pyramid}


def cmd_generate(a) -> dict:
    size = tuple(a.size)
    voxel = tuple(a.voxel) if a.voxel else (1.0 / max(size),) * 3
    fbm = fbm_desc(seed=a.seed, octaves=a.octaves, lacunarity=a.lacunarity, gain=a.gain,
                   base_frequency=a.frequency)
    desc = grid_desc(size, voxel)
    if a.device:
        with Context(a.gpu) as ctx:
            ctx.grid_generate(desc, fbm, _abi.PREC_FP32)
            data = ctx.grid_read_dense()
    else:
        data = fbm_fill_host(size, fbm)
    xyz_write(a.output, desc, data)
    return {"wrote": a.output, "size": list(size), "voxel_size": list(voxel), "max": float(data.max()),
            "mean": float(data.mean())}


def cmd_info(a) -> dict:
    desc, data = xyz_read(a.input)
    size = tuple(desc.size)
    return {"file": a.input, "size": list(size), "voxel_size": list(desc.voxel_size[:]),
            "majorant": float(data.max()), "min": float(data.min()), "mean": float(data.mean()),
            "nonzero_fraction": float(np.count_nonzero(data) / max(data.size, 1)),
            "device_bytes": {p: device_bytes(size, p)["total"] for p in PRECISIONS}}


def cmd_convert(a) -> dict:
    desc, data = xyz_read(a.input)
    with Context(a.gpu) as ctx:
        ctx.grid_upload(desc, data, PRECISIONS[a.precision])
        stored = ctx.grid_read_dense()
    xyz_write(a.output, desc, stored)
    err = np.abs(stored.astype(np.float64) - data)
    mx = float(data.max()) or 1.0
    return {"wrote": a.output, "precision": a.precision, "max_abs_error": float(err.max()),
            "max_error_over_majorant": float(err.max() / mx), "rms_error": float(np.sqrt(np.mean(err ** 2)))}


def cmd_slice(a) -> dict:
    desc, data = xyz_read(a.input)  # [Z, Y, X]
    axis = "zyx".index(a.axis)
    img = np.take(data, a.index, axis=axis)
    hi = float(img.max()) if a.scale <= 0 else a.scale
    g = np.clip(img / (hi or 1.0), 0.0, 1.0)
    g8 = (g * 255.0 + 0.5).astype(np.uint8)
    rgba = np.stack([g8, g8, g8, np.full_like(g8, 255)], axis=-1)
    write_png(a.output, rgba)  # rows: the slower of the two remaining axes
    return {"wrote": a.output, "axis": a.axis, "index": a.index, "shape": list(img.shape), "scale": hi}


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="python -m vcr.grid_tool", description=__doc__.split("\n\n")[0])
    sub = ap.add_subparsers(dest="cmd", required=True)
    g = sub.add_parser("generate", help="seeded fBm cloud -> .xyz")
    g.add_argument("--size", type=int, nargs=3, required=True, metavar=("X", "Y", "Z"))
    g.add_argument("--voxel", type=float, nargs=3, metavar=("VX", "VY", "VZ"),
                   help="voxel size (default: the longest axis spans 1)")
    g.add_argument("--seed", type=int, default=1)
    g.add_argument("--octaves", type=int, default=6)
    g.add_argument("--lacunarity", type=float, default=2.0)
    g.add_argument("--gain", type=float, default=0.5)
    g.add_argument("--frequency", type=float, default=4.0, help="base noise frequency over the longest axis")
    g.add_argument("--device", action="store_true", help="generate on the GPU")
    g.add_argument("--gpu", type=int, default=0)
    g.add_argument("-o", "--output", required=True)
    i = sub.add_parser("info", help="header, majorant, statistics, device bytes per precision")
    i.add_argument("input")
    c = sub.add_parser("convert", help="store as FP32 / FP16 / BF16 bricks and write back what is sampled")
    c.add_argument("input")
    c.add_argument("--precision", choices=sorted(PRECISIONS), default="fp16")
    c.add_argument("--gpu", type=int, default=0)
    c.add_argument("-o", "--output", required=True)
    s = sub.add_parser("slice", help="one axis-aligned slice as a grey PNG")
    s.add_argument("input")
    s.add_argument("--axis", choices=["x", "y", "z"], default="z")
    s.add_argument("--index", type=int, required=True)
    s.add_argument("--scale", type=float, default=0.0, help="density shown as white (default: the slice max)")
    s.add_argument("-o", "--output", required=True)
    a = ap.parse_args(argv)
    out = {"generate": cmd_generate, "info": cmd_info, "convert": cmd_convert, "slice": cmd_slice}[a.cmd](a)
    print(json.dumps(out))
    return 0


if __name__ == "__main__":
    sys.exit(main())
