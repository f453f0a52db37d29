"""Mechanical GLSL -> C++ rewrite of a line range of one reference shader file.

TEST INFRASTRUCTURE (oracle side, run by oracle/Makefile target `ref`): the
output is compiled into oracle/_ref/ref_shader_pin together with
oracle/ref_shim/glsl_shim.h, so that the reference's own shader functions can
be compared with the oracle's restatement of them. Nothing of the reference is
copied into the repository: the rewrite runs on the checkout at build time and
writes only under oracle/_ref/.

The rewrite changes syntax only, never arithmetic:
  - parameter qualifiers: `inout T x` / `out T x` -> `T& x`, `in T x` -> `T x`;
  - swizzles `.xyz` / `.yzx` / ... (2-4 of xyzw) -> member calls `.xyz()`;
  - unsuffixed floating literals get an `f` (GLSL literals are float, C++'s
    double): `0.5` -> `0.5f`;
  - `precise` and loop attributes (`[[unroll]]`) are dropped (the shim is
    compiled without contraction, which is what `precise` asks for).

usage: python glsl_to_cpp.py <shader file> <first line> <last line> <out file>
"""
import os
import re
import sys

_QUAL = re.compile(r"(?<=[(,])(\s*)(inout|out|in)\s+(\w+)\s+(\w+)")
_SWIZ = re.compile(r"\.([xyzw]{2,4})\b(?!\s*\()")
_FLOAT = re.compile(r"(?<![\w.])(\d+\.\d*|\.\d+)([eE][+-]?\d+)?(?![fF\w.])")


def _qualifier(m):
    ws, qual, typ, name = m.groups()
    return f"{ws}{typ}{'&' if qual in ('inout', 'out') else ''} {name}"


def rewrite_line(line: str) -> str:
    code, sep, comment = line.partition("//")
    code = re.sub(r"\bprecise\s+", "", code)
    code = re.sub(r"\[\[\s*\w+\s*\]\]", "", code)
    code = _QUAL.sub(_qualifier, code)
    code = _SWIZ.sub(lambda m: f".{m.group(1)}()", code)
    code = _FLOAT.sub(lambda m: m.group(0) + "f", code)
    return code + sep + comment


def main(argv) -> int:
    if len(argv) != 5:
        print(__doc__, file=sys.stderr)
        return 2
    src, first, last, out = argv[1], int(argv[2]), int(argv[3]), argv[4]
    with open(src) as f:
        lines = f.read().split("\n")
    body = [rewrite_line(line) for line in lines[first - 1:last]]
    os.makedirs(os.path.dirname(os.path.abspath(out)), exist_ok=True)
    with open(out, "w") as f:
        f.write(f"// generated by oracle/glsl_to_cpp.py from {os.path.basename(src)}:{first}-{last}\n")
        f.write(f'#line {first} "{os.path.basename(src)}"\n')
        f.write("\n".join(body) + "\n")
    return 0


if __name__ == "__main__":
    raise SystemExit(main(sys.argv))
