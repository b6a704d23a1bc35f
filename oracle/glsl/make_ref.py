"""Builds oracle/_ref/libglslref.so from the reference's own GLSL helpers --
TEST INFRASTRUCTURE ONLY (the recipe; run by tests/golden/gen_glsl_goldens.py).

The engine's shading math and its software scene traversal live in GLSL
include files that need no graphics API: data/shader/brdf/{brdf,brdfEval,
brdfSample,surface}.hsh, raytracer/{lights,intersections,structures,bvh,
direct,buffers,texture}.hsh, common/{random,utility,PI,material,packing}.hsh.
This recipe reads them where they lie in the
reference tree (unchanged on disk), flattens their `#include <...>` lines the
way the engine's shader loader does (relative to the including file, each
file once), and makes the GLSL parse as C++ with the vector types of
glsl.hpp.  The text of every function is kept; only these mechanical,
language-level adjustments are applied:

  * `#extension` lines are dropped;
  * `in T x` / `out T x` / `inout T x` parameters become `T x` / `T& x` /
    `T& x` (GLSL's copy-out semantics, expressed as C++ references);
  * float literals get an `f` suffix (a GLSL float literal is single
    precision, a C++ one double);
  * an array constructor `T[N](a, b, ...)` becomes the brace list `{a, b, ...}`;
  * resource declarations (`layout(...)`, storage `buffer` blocks, `uniform`
    blocks and variables, `shared` arrays) become plain globals: a buffer
    block's runtime-sized arrays become pointers, an array of buffer blocks
    (one per mesh under bindless resources) a table of such pointers, which
    glsl_capi.cpp points at the caller's scene;
  * the engine's globals.hsh (uniform blocks and bindless textures) is
    replaced by the resources the helpers name: the DFG lookup texture and
    the bindless texture table with its sampler.

Each program's flattened source goes to oracle/_ref/<program>.inc (every
program in a namespace of its own, the compute shaders' `main` renamed
<namespace>_main; rayGen.csh, rayHit.csh and rtao.csh, the last twice: with
and without OPACITY_CHECK), and glsl_capi.cpp includes them all; it is
compiled (-O2 -ffp-contract=off) into oracle/_ref/libglslref.so.  Usage: python make_ref.py [REFERENCE_ROOT]
"""
from __future__ import annotations

import re
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ORACLE = HERE.parent
OUT_DIR = ORACLE / "_ref"
# Programs, each in a namespace of its own (a compute shader brings its own
# `main`, uniform block and buffers; and the shim's types live in the global
# namespace, so argument-dependent lookup must not see two programs'
# functions): the helpers, the path tracer's ray generation and its hit
# shader, and the ambient-occlusion pass in its two variants (the engine
# compiles rtao.csh with or without OPACITY_CHECK, AORenderer.cpp:89).
# Entries: namespace, files, macros defined for the program alone.
PROGRAMS = {
    "glsl_ref": ("aeg_glsl", ["brdf/brdfSample.hsh", "raytracer/lights.hsh", "raytracer/intersections.hsh",
                        "raytracer/bvh.hsh", "raytracer/direct.hsh"], []),
    "glsl_raygen": ("aeg_raygen", ["pathtracer/rayGen.csh"], []),
    "glsl_pt": ("aeg_pt", ["pathtracer/rayHit.csh"], []),
    "glsl_rtao": ("aeg_rtao", ["ao/rtao.csh"], []),
    "glsl_rtao_opacity": ("aeg_rtao_opacity", ["ao/rtao.csh"], ["OPACITY_CHECK"]),
    "glsl_rtr": ("aeg_rtr", ["reflection/rtreflection.csh"], []),
    "glsl_rtr_opacity": ("aeg_rtr_opacity", ["reflection/rtreflection.csh"], ["OPACITY_CHECK"]),
    "glsl_rtgi": ("aeg_rtgi", ["rtgi/rtgi.csh"], []),
    "glsl_rtgi_opacity": ("aeg_rtgi_opacity", ["rtgi/rtgi.csh"], ["OPACITY_CHECK"]),
    "glsl_ddgi_raygen": ("aeg_ddgi_rg", ["ddgi/rayGen.csh"], []),
    "glsl_ddgi": ("aeg_ddgi", ["ddgi/rayHit.csh"], []),
}
# The engine compiles its shaders with bindless resources (AE_BINDLESS: one
# buffer per mesh) and, where registers allow, the traversal stack in local
# memory (LOCAL_STACK, bvh.hsh:39-42); compute shaders see one invocation.
PREAMBLE = "#define AE_BINDLESS\n#define LOCAL_STACK\n"
# the compute shaders' work-group sizes (pathtracer/rayGen.csh: local_size
# 8 x 8; rtao.csh, rtreflection.csh, rtgi.csh: 8 x 4; ddgi/rayGen.csh and
# ddgi/rayHit.csh: 32)
WORKGROUP = {"aeg_raygen": "static const uvec3 gl_WorkGroupSize(8u, 8u, 1u);\n",
             "aeg_rtao": "static const uvec3 gl_WorkGroupSize(8u, 4u, 1u);\n",
             "aeg_rtao_opacity": "static const uvec3 gl_WorkGroupSize(8u, 4u, 1u);\n",
             "aeg_rtr": "static const uvec3 gl_WorkGroupSize(8u, 4u, 1u);\n",
             "aeg_rtr_opacity": "static const uvec3 gl_WorkGroupSize(8u, 4u, 1u);\n",
             "aeg_rtgi": "static const uvec3 gl_WorkGroupSize(8u, 4u, 1u);\n",
             "aeg_rtgi_opacity": "static const uvec3 gl_WorkGroupSize(8u, 4u, 1u);\n",
             "aeg_ddgi_rg": "static const uvec3 gl_WorkGroupSize(32u, 1u, 1u);\n",
             "aeg_ddgi": "static const uvec3 gl_WorkGroupSize(32u, 1u, 1u);\n"}
GLOBALS_STUB = ("static glsl_sampler2D dfgTexture;\n"
                "static glsl_texture2D* bindlessTextures = nullptr;\n"
                "static glsl_sampler bindlessSampler;\n"
                # the members of globals.hsh's GlobalBuffer that rayGen.csh,
                # rtao.csh and convert.hsh read
                "struct GlobalBufferStub { vec2 jitterCurrent; vec4 cameraLocation; mat4 ivMatrix; "
                "mat4 ipMatrix; uint frameCount; };\n"
                "static GlobalBufferStub globalData;\n")

_INCLUDE = re.compile(r'^\s*#include\s*<([^>]+)>\s*$')
_FLOAT = re.compile(r'(?<![\w.])((?:\d+\.\d*|\.\d+)(?:[eE][+-]?\d+)?|\d+[eE][+-]?\d+)(?![\w.])')
_QUAL = re.compile(r'\b(inout|out|in)[ \t]+([A-Za-z_]\w*)[ \t]+([A-Za-z_]\w*)')
_LAYOUT = re.compile(r'\blayout\s*\([^)]*\)\s*')
_BUFFER = re.compile(r'\bbuffer\s+\w+\s*\{([^}]*)\}\s*;', re.S)
_BUFFER_ARRAY = re.compile(r'\bbuffer\s+(\w+)\s*\{([^}]*)\}\s*(\w+)\s*\[([^\]]*)\]\s*;', re.S)
_UNIFORM_BLOCK = re.compile(r'\buniform\s+(\w+)\s*\{')
_UNIFORM_VAR = re.compile(r'^(\s*)(?:readonly\s+|writeonly\s+)*uniform\s+(\w+\s+\w+(?:\s*\[[^\]]*\])?\s*;)', re.M)
_SHARED = re.compile(r'^(\s*)shared\s+', re.M)
_LAYOUT_IN = re.compile(r'^\s*in\s*;\s*$', re.M)
_ARRAY_CTOR = re.compile(r'=\s*\w+\s*\[\s*\d*\s*\]\s*\((.*?)\);', re.S)


def _flatten(path: Path, seen: set, shader_root: Path) -> str:
    path = path.resolve()
    if path in seen:
        return ""
    seen.add(path)
    if path == (shader_root / "globals.hsh").resolve():
        return GLOBALS_STUB
    out = []
    for line in path.read_text().splitlines():
        m = _INCLUDE.match(line)
        if m:
            out.append(_flatten(path.parent / m.group(1), seen, shader_root))
        elif line.lstrip().startswith("#extension"):
            continue
        else:
            out.append(line)
    return "\n".join(out) + "\n"


def _buffer_to_globals(m: re.Match) -> str:
    decls = []
    for d in m.group(1).split(";"):
        d = d.strip()
        if not d:
            continue
        arr = re.match(r'(\w+)\s+(\w+)\s*\[\s*\]$', d)
        decls.append(f"static {arr.group(1)}* {arr.group(2)} = nullptr;" if arr else f"static {d};")
    return "\n".join(decls)


def _buffer_array(m: re.Match) -> str:
    # one block per mesh (bindless): a table of per-mesh pointers
    fields = []
    for d in m.group(2).split(";"):
        d = d.strip()
        if d:
            arr = re.match(r'(\w+)\s+(\w+)\s*\[\s*\]$', d)
            fields.append(f"{arr.group(1)}* {arr.group(2)} = nullptr;" if arr else f"{d};")
    return f"struct {m.group(1)} {{ {' '.join(fields)} }};\nstatic {m.group(1)} {m.group(3)}[{m.group(4)}];"


def to_cpp(src: str) -> str:
    def qual(m):
        return f"{m.group(2)}& {m.group(3)}" if m.group(1) in ("inout", "out") else f"{m.group(2)} {m.group(3)}"
    src = _QUAL.sub(qual, src)
    src = _LAYOUT.sub("", src)
    src = _LAYOUT_IN.sub("", src)
    src = _BUFFER_ARRAY.sub(_buffer_array, src)
    src = _BUFFER.sub(_buffer_to_globals, src)
    src = _UNIFORM_BLOCK.sub(lambda m: f"struct {m.group(1)} {{", src)
    src = _UNIFORM_VAR.sub(lambda m: f"{m.group(1)}static {m.group(2)}", src)
    src = _SHARED.sub(lambda m: f"{m.group(1)}static ", src)
    # an array constructor `T[N](a, b, ...)` initialises like a brace list
    src = _ARRAY_CTOR.sub(lambda m: "= {" + m.group(1) + "};", src)
    src = _FLOAT.sub(lambda m: m.group(1) + "f", src)
    return src


def build(reference_root: Path) -> Path:
    shader_root = reference_root / "data" / "shader"
    OUT_DIR.mkdir(exist_ok=True)
    header = "// generated by oracle/glsl/make_ref.py from the reference's shader files; do not edit\n"
    for name, (ns, files, macros) in PROGRAMS.items():
        seen: set = set()
        body = to_cpp("".join(_flatten(shader_root / f, seen, shader_root) for f in files))
        # the program's entry point becomes <namespace>_main
        body = (f"namespace {ns} {{\n#define main {ns}_main\n" + "".join(f"#define {m}\n" for m in macros) +
                WORKGROUP.get(ns, "") + body + "".join(f"\n#undef {m}" for m in macros) +
                f"\n#undef main\n}}  // namespace {ns}\n")
        (OUT_DIR / f"{name}.inc").write_text(header + PREAMBLE + body)
    lib = OUT_DIR / "libglslref.so"
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-fno-builtin",
           "-w", f"-I{HERE}", f"-I{OUT_DIR}", str(HERE / "glsl_capi.cpp"), "-o", str(lib)]
    subprocess.run(cmd, check=True)
    return lib


if __name__ == "__main__":
    root = Path(sys.argv[1]) if len(sys.argv) > 1 else None
    if root is None:
        sys.path.insert(0, str(ORACLE))
        import pyoracle
        root = pyoracle.REFERENCE_ROOT
    print(build(root))
