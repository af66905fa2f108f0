"""Alembic fixtures for tests/test_alembic.py.

Builds oracle/_ref/abc_tool (the reference's vendored Alembic SDK and its
Houdini reader, libs/abc and libs/houdini_alembic, compiled from their
sources), writes the synthetic scenes with the SDK's writer, and stores what
the reference reader returns for them (``abc_tool dump``) as JSON:

  basic.abc   transform chain (translate / rotate / scale, axis-angle, matrix
              op), triangle meshes with every material column, a quad mesh, a
              hidden and a "visible = 1" parent, spheres, the ImageEnvmap
              point, a camera with resx / resy -> basic.json
  render.abc  a floor of random materials, a light panel, spheres, camera
              -> render.json
  anim.abc    three frames of a transform and vertex positions
              -> anim_f{0,1,2,5}.json (frame 5 clamps to the last sample)
  badmat.abc  a mesh whose material names an unregistered class

and writes the Radiance .hdr images the tests load: sky_tiny.hdr (16 x 8,
run-length encoded scanlines; the basic scene's envmap) and flat_tiny.hdr
(4 x 2, flat RGBE).  Needs the reference sources (run in the development
container); the GPU machines use the committed files.
"""
from __future__ import annotations

import math
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
OUT = HERE / "alembic"
ROOT = HERE.parent.parent


def rgbe(rgb: np.ndarray) -> np.ndarray:
    """Float RGB -> RGBE bytes (shared exponent of the largest channel)."""
    out = np.zeros(rgb.shape[:-1] + (4,), np.uint8)
    for idx in np.ndindex(rgb.shape[:-1]):
        v = float(rgb[idx].max())
        if v < 1e-32:
            continue
        m, e = math.frexp(v)
        scale = m * 256.0 / v
        out[idx][:3] = np.minimum(np.floor(rgb[idx] * scale), 255).astype(np.uint8)
        out[idx][3] = e + 128
    return out


def write_hdr(path: Path, rgb: np.ndarray, rle: bool) -> None:
    h, w = rgb.shape[:2]
    px = rgbe(rgb)
    data = bytearray(b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\nEXPOSURE=1.0\n\n")
    data += f"-Y {h} +X {w}\n".encode()
    for y in range(h):
        if not rle:
            data += px[y].tobytes()
            continue
        data += bytes([2, 2, w >> 8, w & 255])
        for c in range(4):
            ch = px[y, :, c]
            x = 0
            while x < w:  # runs of equal bytes where they pay, literals elsewhere
                run = 1
                while x + run < w and run < 127 and ch[x + run] == ch[x]:
                    run += 1
                if run >= 3:
                    data += bytes([128 + run, int(ch[x])])
                    x += run
                else:
                    lit = 1
                    while x + lit < w and lit < 128:
                        nxt = 1
                        while x + lit + nxt < w and ch[x + lit + nxt] == ch[x + lit]:
                            nxt += 1
                        if nxt >= 3:
                            break
                        lit += 1
                    data += bytes([lit]) + ch[x:x + lit].tobytes()
                    x += lit
    path.write_bytes(bytes(data))


def main() -> None:
    sys.path.insert(0, str(ROOT))
    from oracle import build_oracle
    tool = build_oracle.build_abc_tool()
    if tool is None:
        raise SystemExit("the reference sources are needed to regenerate the Alembic fixtures")
    OUT.mkdir(parents=True, exist_ok=True)

    def run(*args) -> str:
        return subprocess.run([str(tool), *map(str, args)], check=True, capture_output=True, text=True).stdout

    for scene in ("basic", "render", "anim", "badmat"):
        run("write", OUT / f"{scene}.abc", scene)
    (OUT / "basic.json").write_text(run("dump", OUT / "basic.abc", 0))
    (OUT / "render.json").write_text(run("dump", OUT / "render.abc", 0))
    for f in (0, 1, 2, 5):
        (OUT / f"anim_f{f}.json").write_text(run("dump", OUT / "anim.abc", f))
    rng = np.random.default_rng(5)
    sky = rng.uniform(0.0, 3.0, (8, 16, 3)).astype(np.float32)
    sky[2:4, 5:12] = [0.5, 0.7, 1.0]          # runs, for the run-length encoder
    sky[1, 3] = [400.0, 380.0, 300.0]         # above the scene's clamp of 50
    write_hdr(OUT / "sky_tiny.hdr", sky, rle=True)
    write_hdr(OUT / "flat_tiny.hdr", rng.uniform(0.0, 2.0, (2, 4, 3)).astype(np.float32), rle=False)
    print("wrote", sorted(p.name for p in OUT.iterdir()))


if __name__ == "__main__":
    main()
