"""Regenerate ``anorms_table.h`` from the reference's 162 sky directions.

The table is data, not code: ``vmath/constants.go:21-184`` of the reference
lists ``NUMVERTEXNORMALS = 162`` unit vectors (``Anorms``) that
``rad/lightmap/lightmap.go:425-451`` (``CanLeafTraceToSky``) sweeps when it
looks for sky.  This script parses the Go literals and writes them out as a C
array with the decimal text unchanged, so a C compiler rounds each literal to
float32 exactly as Go's constant conversion does.

Usage:  python vrad_gb300/csrc/gen_anorms.py <reference checkout>/vmath/constants.go
The generated header is committed; the GPU build never needs the reference.
"""
import re
import sys
from pathlib import Path


def parse(go_source: str):
    body = go_source[go_source.index("var Anorms"):]
    body = body[: body.index("\n}") + 2]
    vecs = re.findall(r"mgl32\.Vec3\{\s*([-0-9.eE]+)\s*,\s*([-0-9.eE]+)\s*,\s*([-0-9.eE]+)\s*\}", body)
    if len(vecs) != 162:
        raise SystemExit(f"expected 162 directions, found {len(vecs)}")
    return vecs


def render(vecs) -> str:
    lines = [
        "/* Generated by gen_anorms.py from the reference's vmath/constants.go:21-184",
        " * (Anorms, NUMVERTEXNORMALS = 162).  Do not edit by hand. */",
        "#ifndef VRG_ANORMS_TABLE_H",
        "#define VRG_ANORMS_TABLE_H",
        "#define VRG_NUM_ANORMS 162",
        "#define VRG_ANORMS_INIT { \\",
    ]
    for i, (x, y, z) in enumerate(vecs):
        sep = "," if i + 1 < len(vecs) else ""
        lines.append(f"  {x}f, {y}f, {z}f{sep} \\")
    lines.append("}")
    lines.append("#endif")
    return "\n".join(lines) + "\n"


def main():
    if len(sys.argv) != 2:
        raise SystemExit("usage: gen_anorms.py <path to the reference's vmath/constants.go>")
    src = Path(sys.argv[1])
    out = Path(__file__).with_name("anorms_table.h")
    out.write_text(render(parse(src.read_text())))
    print(f"wrote {out}")


if __name__ == "__main__":
    main()
