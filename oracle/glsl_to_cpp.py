"""Rewrites the declarations of a GLSL compute shader so that its code
compiles as C++ against oracle/glsl_shim/glsl.hpp (test infrastructure
only; the output goes to oracle/_ref/ and is never committed).

Usage: python glsl_to_cpp.py <shader.glsl> <out.inc>

Only declaration syntax changes; every function body is kept as written:
  * '#version' lines are dropped;
  * 'layout(local_size_x = X, local_size_y = Y, local_size_z = Z) in;' becomes
    the constant gl_WorkGroupSize = uvec3(X, Y, Z);
  * other 'layout(...)' qualifiers and 'readonly' are dropped, 'uniform'
    declarations become plain globals (the driver sets them);
  * a shader storage block 'buffer Name { T member[]; };' becomes a global
    pointer 'T* member' (the driver points it at the caller's records);
  * 'inout T name' parameters become references 'T& name';
  * 'void main()' becomes 'void shader_main()';
  * a local struct variable declared without initialiser ('Hit hit;')
    is value-initialised ('Hit hit{};'), so its unwritten fields are the
    shim's defaults (NaN floats, zero integers) rather than indeterminate.
The written file names its source and states that it was generated.
"""
from __future__ import annotations

import re
import sys


def convert(src: str) -> str:
    out = src
    out = re.sub(r"^\s*#version[^\n]*\n", "", out, flags=re.M)
    m = re.search(r"layout\s*\(\s*local_size_x\s*=\s*(\d+)\s*,\s*local_size_y\s*=\s*(\d+)\s*,"
                  r"\s*local_size_z\s*=\s*(\d+)\s*\)\s*in\s*;", out)
    if not m:
        raise SystemExit("no local_size layout found")
    out = out.replace(m.group(0), f"const uvec3 gl_WorkGroupSize = uvec3({m.group(1)}, {m.group(2)}, {m.group(3)});")
    out = re.sub(r"(?:readonly\s+)?buffer\s+\w+\s*\{\s*(\w+)\s+(\w+)\s*\[\s*\]\s*;\s*\}\s*;",
                 r"\1* \2 = nullptr;", out)
    out = re.sub(r"layout\s*\([^)]*\)\s*", "", out)
    out = re.sub(r"\breadonly\s+", "", out)
    out = re.sub(r"^(\s*)uniform\s+", r"\1", out, flags=re.M)
    out = re.sub(r"\binout\s+(\w+)\s+", r"\1& ", out)
    out = re.sub(r"\bvoid\s+main\s*\(\s*\)", "void shader_main()", out)
    structs = set(re.findall(r"\bstruct\s+(\w+)", out))
    if structs:
        pat = r"^(\s+)(" + "|".join(sorted(structs)) + r")\s+(\w+)\s*;"
        out = re.sub(pat, r"\1\2 \3{};", out, flags=re.M)
    return out


def main() -> None:
    src_path, out_path = sys.argv[1], sys.argv[2]
    with open(src_path) as f:
        src = f.read()
    body = convert(src)
    with open(out_path, "w") as f:
        f.write(f"// Generated by oracle/glsl_to_cpp.py from {src_path}; do not edit or commit.\n")
        f.write(body)


if __name__ == "__main__":
    main()
