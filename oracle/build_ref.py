"""Compile the reference's own GLSL compute shaders as C++ into oracle/_ref/ (test infrastructure).

The reference's hot path is five GLSL 4.3 compute shaders (paths inside the reference project):
  data/shaders/gi/vpl_processor.comp, data/shaders/ism/ism.comp, data/shaders/ism/pull.comp,
  data/shaders/ism/push.comp, data/shaders/gi/final_gathering.comp
and its clustered culling two more: data/shaders/clustered_shading/clustering.comp and
  data/shaders/clustered_shading/light_lists.comp
plus their includes (common/floatpacking.glsl, common/random.glsl, common/reprojection.glsl,
ism/ism_utils.glsl). This recipe reads them where they lie under the reference root (REF below), applies a fixed
list of mechanical GLSL -> C++ rewrites (below), and compiles the result together with
oracle/ref_shim.hpp (GLSL types and built-ins) and oracle/ref_harness.cpp (images, buffers,
dispatch, work-group fibers) into oracle/_ref/libref.so. No reference source is copied into the
repository; the generated files live only in oracle/_ref/ (git-ignored).

Rewrites (nothing else is changed):
  1. drop `#version` / `#extension` lines; inline `#include </data/shaders/...>` (what
     GL_ARB_shading_language_include does);
  2. variants: `#define LEVEL_ZERO` -> `#undef LEVEL_ZERO` for the non-level-zero pull/push programs,
     exactly the replacement ImperfectShadowmap.cpp:52-60 applies;
  3. drop the work-group size declaration `layout(local_size_...) in;` (the harness passes it);
  4. float literals get an `f` suffix (GLSL literals are single precision);
  5. GLSL array syntax `T[N] name` -> `T name[N]`;
  6. swizzles `.xy/.xyz/.rgb/.rg` -> accessor calls, `.r/.g/.b/.a` -> `.x/.y/.z/.w`;
  7. parameter qualifier `in` dropped; memory qualifiers (restrict, readonly, writeonly, coherent)
     dropped;
  8. `uniform T name [= v];` -> a member read from the harness's bindings (default v);
     (and for the fragment shader gi_blur.frag: `inout` parameters -> references, stage `in`/`out`
     variables -> members the harness sets and reads; the X and Y programs are the reference's own
     DIRECTION replacements, GIStage.cpp:444-449)
     interface blocks `layout(...) uniform|buffer Name { T member[...]; };` -> members bound to
     harness arrays; `shared T name[N];` -> a view of the work group's shared arena.
The shaders are wrapped as C++ structs (globals -> members, main() -> member function).

On a host without the reference sources, the generated files in oracle/_ref/gen (which travel
with the working tree) are compiled instead; with neither, build_if_reference_present() does
nothing.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# Root of the reference project: MLGI_REFERENCE_ROOT, or `--reference <dir>` on the command line,
# else where this build reads it.
REF = os.environ.get("MLGI_REFERENCE_ROOT", "/root/reference")
if "--reference" in sys.argv[:-1]:
    REF = sys.argv[sys.argv.index("--reference") + 1]
OUT = os.path.join(HERE, "_ref")
GEN = os.path.join(OUT, "gen")
LIB = os.path.join(OUT, "libref.so")

SHADERS = {
    # struct name: (shader path, replacements applied before the rewrite)
    "Ref_vpl_processor": ("data/shaders/gi/vpl_processor.comp", []),
    "Ref_ism": ("data/shaders/ism/ism.comp", []),
    "Ref_pull_L0": ("data/shaders/ism/pull.comp", []),
    "Ref_pull": ("data/shaders/ism/pull.comp", [("#define LEVEL_ZERO", "#undef LEVEL_ZERO")]),
    "Ref_push_L0": ("data/shaders/ism/push.comp", []),
    "Ref_push": ("data/shaders/ism/push.comp", [("#define LEVEL_ZERO", "#undef LEVEL_ZERO")]),
    "Ref_final_gathering": ("data/shaders/gi/final_gathering.comp", []),
    "Ref_clustering": ("data/shaders/clustered_shading/clustering.comp", []),
    # the X and Y programs GIStage.cpp:444-449 builds from the fragment shader by global replacement
    "Ref_gi_blur_x": ("data/shaders/gi/gi_blur.frag", [("#define DIRECTION ivec2(0,0)", "#define DIRECTION ivec2(1,0)")]),
    "Ref_gi_blur_y": ("data/shaders/gi/gi_blur.frag", [("#define DIRECTION ivec2(0,0)", "#define DIRECTION ivec2(0,1)")]),
    "Ref_light_lists": ("data/shaders/clustered_shading/light_lists.comp", []),
}

GLSL_TYPES = ("float", "int", "uint", "bool", "vec2", "vec3", "vec4", "ivec2", "ivec3", "ivec4", "uvec2",
              "uvec3", "uvec4", "mat3", "mat4")


def read_shader(rel: str, seen=None) -> str:
    seen = set() if seen is None else seen
    src = open(os.path.join(REF, rel)).read()
    out = []
    for line in src.splitlines():
        s = line.strip()
        if s.startswith("#version") or s.startswith("#extension"):
            continue
        m = re.match(r"#include\s*</?(.*?)>", s)
        if m:
            inc = m.group(1)
            if inc not in seen:
                seen.add(inc)
                out.append(read_shader(inc, seen))
            continue
        out.append(line)
    return "\n".join(out)


def rewrite(src: str) -> str:
    # 3. work-group size declaration
    src = re.sub(r"layout\s*\(\s*local_size[^)]*\)\s*in\s*;", "", src)
    # 4. float literals
    src = re.sub(r"(?<![\w.])(\d+\.\d*(?:[eE][+-]?\d+)?|\.\d+(?:[eE][+-]?\d+)?|\d+[eE][+-]?\d+)(?![\w.])", r"\1f", src)
    # 8a. interface blocks
    def block(m):
        members = []
        for decl in m.group(3).split(";"):
            decl = decl.strip()
            if not decl:
                continue
            dm = re.match(r"(\w+)\s*\[[^\]]*\]\s+(\w+)$", decl) or re.match(r"(\w+)\s+(\w+)\s*\[[^\]]*\]$", decl)
            if dm:
                members.append(f'{dm.group(1)}* {dm.group(2)} = buf<{dm.group(1)}>("{dm.group(2)}");')
                continue
            sm = re.match(r"(\w+)\s+(\w+)$", decl)
            if sm:
                members.append(f'{sm.group(1)}& {sm.group(2)} = *buf<{sm.group(1)}>("{sm.group(2)}");')
                continue
            raise ValueError("unhandled block member: " + decl)
        return "\n".join(members)
    src = re.sub(r"layout\s*\([^)]*\)\s*(uniform|buffer)\s+(\w+)\s*\{(.*?)\}\s*;", block, src, flags=re.S)
    # 7. qualifiers
    src = re.sub(r"\b(restrict|readonly|writeonly|coherent)\b", "", src)
    src = re.sub(r"layout\s*\([^)]*\)\s*", "", src)
    # 8b. uniforms
    def uniform(m):
        t, n, d = m.group(1), m.group(2), m.group(3)
        return f'{t} {n} = uni<{t}>("{n}"' + (f", {d.strip()}" if d else "") + ");"
    src = re.sub(r"\buniform\s+(\w+)\s+(\w+)\s*(?:=\s*([^;]+))?;", uniform, src)
    # 8c. shared declarations (GLSL array syntax or C syntax or scalar)
    def shared(m):
        body = m.group(1).strip()
        am = re.match(r"(\w+)\s*\[([^\]]+)\]\s+(\w+)$", body) or re.match(r"(\w+)\s+(\w+)\s*\[([^\]]+)\]$", body)
        if am:
            if re.match(r"(\w+)\s*\[", body):
                t, n, name = am.group(1), am.group(2), am.group(3)
            else:
                t, name, n = am.group(1), am.group(2), am.group(3)
            return f'{t}* {name} = shared_mem<{t}>("{name}", {n});'
        sm = re.match(r"(\w+)\s+(\w+)$", body)
        return f'{sm.group(1)}& {sm.group(2)} = *shared_mem<{sm.group(1)}>("{sm.group(2)}", 1);'
    src = re.sub(r"^\s*shared\s+([^;]+);", shared, src, flags=re.M)
    # 5. GLSL array syntax for locals and globals
    types = "|".join(GLSL_TYPES)
    src = re.sub(r"\b(" + types + r")\s*\[([^\]]+)\]\s+(\w+)", r"\1 \3[\2]", src)
    # 6. swizzles
    src = re.sub(r"\.(xyz|xy|rgb|rg)\b", r".\1()", src)
    src = re.sub(r"\.r\b", ".x", src)
    src = re.sub(r"\.g\b", ".y", src)
    src = re.sub(r"\.b\b", ".z", src)
    src = re.sub(r"\.a\b", ".w", src)
    # 7. parameter qualifier `in`; `inout` parameters become references
    src = re.sub(r"\b(const\s+)?in\s+(\w+\s+\w+\s*[,)])", r"\1\2", src)
    src = re.sub(r"\binout\s+(\w+)\s+(\w+)", r"\1& \2", src)
    # 9. a fragment shader's stage inputs and outputs become members the harness sets and reads
    src = re.sub(r"^\s*(?:in|out)\s+(\w+)\s+(\w+)\s*;", r"\1 \2{};", src, flags=re.M)
    return src


def generate():
    os.makedirs(GEN, exist_ok=True)
    for name, (path, repl) in SHADERS.items():
        src = read_shader(path)
        for a, b in repl:
            src = src.replace(a, b)
        body = rewrite(src)
        # the preprocessor is global: undefine the shader's own macros (include guards, switches)
        macros = sorted(set(re.findall(r"^\s*#\s*define\s+(\w+)", body, flags=re.M)))
        undefs = "\n".join(f"#undef {m}" for m in macros)
        with open(os.path.join(GEN, name + ".inc"), "w") as f:
            f.write(f"// generated by oracle/build_ref.py from {path}\n{body}\n{undefs}\n")


def build(force: bool = False) -> str:
    srcs = [os.path.join(HERE, f) for f in ("ref_harness.cpp", "ref_shim.hpp", "glsl.hpp", "build_ref.py")]
    if os.path.isdir(GEN):
        srcs += [os.path.join(GEN, f) for f in os.listdir(GEN)]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(s) <= os.path.getmtime(LIB) for s in srcs):
        return LIB
    if os.path.isdir(os.path.join(REF, "data", "shaders")):
        generate()
    elif not os.path.isdir(GEN):
        raise RuntimeError("reference shaders not found and no generated sources in oracle/_ref/gen")
    cmd = ["g++", "-O2", "-std=c++20", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
           "-ftrivial-auto-var-init=zero", "-w", f"-I{GEN}", f"-I{HERE}", os.path.join(HERE, "ref_harness.cpp"),
           "-o", LIB + ".tmp"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle/_ref build failed:\n" + " ".join(cmd) + "\n" + r.stdout[-20000:])
    os.replace(LIB + ".tmp", LIB)
    return LIB


def build_if_reference_present():
    """Build from the reference sources here, or from the generated sources that travel with the
    repository to a host without them; do nothing when neither exists."""
    if os.path.isdir(os.path.join(REF, "data", "shaders")) or os.path.isdir(GEN):
        return build()
    return None


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
