"""Field-by-field layout pins between the reference's shaderio structs and the
tc_* structs of include/tc_tessellation.h.

TEST INFRASTRUCTURE (oracle side, run by oracle/Makefile target `ref`): reads
the struct definitions of the reference's shaderio headers (the C++ branch of
every `#ifdef __cplusplus`), and writes, for every field of every pinned
struct, a static_assert that the field has the same offset and size in
shaderio::<S> (the reference header compiled as C++ through
oracle/ref_shim/glsl_shim.h) and in tc_<S>. Compiling the output is the check:
a field missing, renamed, moved or resized fails the build of
oracle/_ref/ref_shader_pin.

usage: python layout_pins.py <out file> <header> [<header> ...]
"""
import os
import re
import sys

# struct -> fields of the reference struct that tc_<struct> leaves out
PINNED = {
    "TessTableEntry": (), "TessellationTable": (), "BBox": (), "Cluster": (), "RenderInstance": (),
    "ClusterInfo": (), "SubTriangleInfo": (), "TessTriangleInfo": (), "ClasBuildInfo": (),
    "TemplateInstantiateInfo": (), "BlasBuildInfo": (), "DispatchIndirectCommand": (),
    "DrawMeshTasksIndirectCommandNV": (), "SceneBuilding": (), "Readback": (),
    # the sky parameters (nvpro_core2's sky_io, not on the tessellation path) end the struct;
    # tc_FrameConstants is the prefix before them
    "FrameConstants": ("skyParams",),
}

_FIELD = re.compile(r"^\s*(?:[\w:]+(?:\s*\([^)]*\))?)\s+(\w+)\s*(?:\[[^\]]*\])?\s*;")


def cpp_branch(text: str) -> str:
    """Keep the __cplusplus side of `#ifdef/#ifndef __cplusplus ... #else ... #endif`."""
    out, stack = [], []
    for line in text.split("\n"):
        s = line.strip()
        if s.startswith("#ifdef __cplusplus"):
            stack.append(True)
            continue
        if s.startswith("#ifndef __cplusplus"):
            stack.append(False)
            continue
        if s.startswith("#if"):
            stack.append(None)
            out.append(line)
            continue
        if s.startswith("#else") and stack and stack[-1] is not None:
            stack[-1] = not stack[-1]
            continue
        if s.startswith("#endif") and stack:
            if stack.pop() is None:
                out.append(line)
            continue
        if all(v is not False for v in stack):
            out.append(line)
    return "\n".join(out)


def struct_fields(text: str, name: str):
    m = re.search(r"\bstruct\s+" + name + r"\s*\{(.*?)\n\};", text, re.S)
    if not m:
        return None
    body = re.sub(r"/\*.*?\*/", "", m.group(1), flags=re.S)
    fields = []
    for line in body.split("\n"):
        line = line.split("//")[0]
        if line.strip().startswith("#"):
            continue
        f = _FIELD.match(line)
        if f:
            fields.append(f.group(1))
    return fields


def main(argv) -> int:
    if len(argv) < 3:
        print(__doc__, file=sys.stderr)
        return 2
    out_path, headers = argv[1], argv[2:]
    text = "\n".join(cpp_branch(open(h).read()) for h in headers)
    lines = ["// generated by oracle/layout_pins.py", "#define TC_PIN_FIELD(S, f) \\",
             "  static_assert(offsetof(shaderio::S, f) == offsetof(tc_##S, f), #S \".\" #f \": offset\"); \\",
             "  static_assert(sizeof(((shaderio::S*)0)->f) == sizeof(((tc_##S*)0)->f), #S \".\" #f \": size\");"]
    count = 0
    for name, skip in PINNED.items():
        fields = struct_fields(text, name)
        if fields is None:
            print(f"struct {name} not found", file=sys.stderr)
            return 1
        kept = [f for f in fields if f not in skip]
        for f in kept:
            lines.append(f"TC_PIN_FIELD({name}, {f})")
        if skip:
            lines.append(f"static_assert(sizeof(tc_{name}) == offsetof(shaderio::{name}, {skip[0]}), "
                         f"\"tc_{name} is the prefix before {skip[0]}\");")
        else:
            lines.append(f"static_assert(sizeof(tc_{name}) == sizeof(shaderio::{name}), \"{name}: size\");")
        lines.append(f"static_assert(alignof(shaderio::{name}) <= alignof(tc_{name}), \"{name}: alignment\");")
        count += len(kept)
    lines.append(f"#define TC_PINNED_FIELDS {count}")
    lines.append(f"#define TC_PINNED_STRUCTS {len(PINNED)}")
    os.makedirs(os.path.dirname(os.path.abspath(out_path)), exist_ok=True)
    with open(out_path, "w") as f:
        f.write("\n".join(lines) + "\n")
    return 0


if __name__ == "__main__":
    raise SystemExit(main(sys.argv))
