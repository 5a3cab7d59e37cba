"""Builds oracle/_ref/: the reference's own GLSL compute shaders for the clustered-shading path (and the
bouncer, depth-pyramid and cluster debug-view shaders), rewritten mechanically into C++ and compiled
for the CPU.  TEST INFRASTRUCTURE ONLY: the tests compare the oracle's C restatement with it.

Nothing of the reference is copied into the repository: this recipe reads the shader files where
they lie in the reference checkout (``VREN_REFERENCE_DIR``, default /root/reference) and writes the
rewritten text only under oracle/_ref/ (git-ignored).  The GLSL semantics the rewritten text relies
on are in oracle/glsl_subset.hpp; the drivers that set up buffers and invocation ids and run the
shaders' main() are in oracle/ref_drivers.cpp.

The rewrite, applied to each shader with its #include files inlined:
  - #version / #extension lines and the local-size layout declaration are dropped;
  - buffer and uniform blocks become namespace-scope variables (unsized arrays become
    glsl::buffer<T>), opaque uniforms become sampler / image objects, `shared` variables static
    ones, other globals thread_local (they are private to an invocation);
  - `out T x` / `inout T x` parameters become `T& x`;
  - float literals get the `f` suffix (GLSL literals are single precision);
  - uint(...), int(...), float(...), bool(...) casts call glsl_uint etc.;
  - scalar locals declared without a value start at zero (GLSL leaves them undefined);
  - `v.xy = e;` becomes `v.set_swz<0, 1>(e);`, swizzles `.xyz` become `.swz<0, 1, 2>()`, single
    components .r .g .b .a become .x .y .z .w;
  - main() becomes shader_main();
  - find_unique_clusters.comp's main() is cut before its first shared-memory store: the per-pixel
    cluster key it computes is returned (the work-group sort and compaction that follow only order
    and deduplicate the keys, which the tests compare as sets);
  - each shader lives in a namespace of its own, its #defines are undefined after it.

Two variants are built from the same text:
  - glsl: the shaders as written, with C library log / tan / pow and a single-precision inverse();
  - canonical: five expressions replaced by the canonical decisions the oracle and the CUDA kernels
    share (each replacement names the decision): the depth slice from the host-built slice table
    instead of floor(log(z / near) / log(a)) (find_unique_clusters.comp:65), the slice bounds
    near * a^k and near * a^(k+1) from the same table instead of pow (clustered_shading.glsl:100-101),
    inverse(projection) and inverse(view) computed once on the host (find_unique_clusters.comp:56,
    clustered_shading.glsl:90, shade.comp:83,88), and the integer texel (x mod W, y mod H) instead of
    sampling at gid / size (find_unique_clusters.comp:50,68; shade.comp:77,89-91).
The tests require the canonical variant to equal the oracle bit for bit and count where the glsl
variant departs from it.
"""
from __future__ import annotations

import os
import re
import shutil
import subprocess
from pathlib import Path

ORACLE_DIR = Path(__file__).resolve().parent
OUT_DIR = ORACLE_DIR / "_ref"
DRIVERS = ORACLE_DIR / "ref_drivers.cpp"
HEADER = ORACLE_DIR / "glsl_subset.hpp"
VARIANTS = ("glsl", "canonical")


def reference_dir() -> Path:
    return Path(os.environ.get("VREN_REFERENCE_DIR", "/root/reference"))


# (namespace, shader path inside the reference, extra #defines, how main() is kept); clustered_shading.glsl
# is an include file that relies on its includer for common.glsl, which is included ahead of it
SHADERS = [
    ("sh_cs", "vren/resources/shaders/clustered_shading.glsl", [], "include"),
    ("sh_view", "vren/resources/shaders/clustered_shading/point_light_position_to_view_space.comp", [], "main"),
    ("sh_morton", "vren/resources/shaders/clustered_shading/discretize_point_light_positions.comp", [], "main"),
    ("sh_leaves", "vren/resources/shaders/clustered_shading/init_light_array_bvh.comp", [], "main"),
    ("sh_unique", "vren/resources/shaders/clustered_shading/find_unique_clusters.comp", [], "key"),
    ("sh_assign_count", "vren/resources/shaders/clustered_shading/assign_lights.comp",
     ["VREN_CLUSTERED_SHADING_LIGHT_ASSIGNMENT_COUNT"], "main"),
    ("sh_assign_write", "vren/resources/shaders/clustered_shading/assign_lights.comp", [], "main"),
    ("sh_shade", "vren/resources/shaders/clustered_shading/shade.comp", [], "main"),
    ("sh_bounce", "vren_demo/resources/shaders/bounce_point_lights.comp", [], "main"),
    ("sh_depth_copy", "vren/resources/shaders/depth_buffer_copy.comp", [], "main"),
    ("sh_depth_reduce", "vren/resources/shaders/depth_buffer_reduce.comp", [], "main"),
    ("sh_show", "vren_demo/resources/shaders/show_clusters.comp", [], "main"),
]

# Canonical decisions: (shader file name, exact text in the reference, replacement).  Every entry must
# be found, so a change in the reference fails the build instead of silently changing the comparison.
CANONICAL = [
    ("find_unique_clusters.comp",
     "uint(floor(log(frag_pos.z / camera_near) / log(1 + (2 * tan(camera_half_fov_y)) / Sy)))",
     "canon_slice(frag_pos.z)"),
    ("find_unique_clusters.comp", "inverse(camera_projection)", "canon_inverse_projection()"),
    ("find_unique_clusters.comp", "texture(u_depth_buffer, frag_coord)", "canon_texel(u_depth_buffer)"),
    ("find_unique_clusters.comp", "texture(gbuffer_normals, frag_coord)", "canon_texel(gbuffer_normals)"),
    ("clustered_shading.glsl", "inverse(camera_proj)", "canon_inverse_projection()"),
    ("clustered_shading.glsl", "camera_near * pow(a, cluster_ijk.z)", "canon_slice_near(cluster_ijk.z)"),
    ("clustered_shading.glsl", "cluster_near * a;", "canon_slice_far(cluster_ijk.z);"),
    ("shade.comp", "inverse(camera_projection)", "canon_inverse_projection()"),
    ("shade.comp", "inverse(camera_view)", "canon_inverse_view()"),
    ("shade.comp", "texture(u_depth_buffer, frag_coord)", "canon_texel(u_depth_buffer)"),
    ("shade.comp", "texture(u_gbuffer_normals, frag_coord)", "canon_texel(u_gbuffer_normals)"),
    ("shade.comp", "texture(u_gbuffer_texcoords, frag_coord)", "canon_texel(u_gbuffer_texcoords)"),
    ("shade.comp", "texture(u_gbuffer_material_indices, frag_coord)", "canon_utexel(u_gbuffer_material_indices)"),
]

SWZ = {"x": 0, "y": 1, "z": 2, "w": 3, "r": 0, "g": 1, "b": 2, "a": 3}


def _inline_includes(path: Path, roots: list[Path], canonical: bool, seen: set) -> str:
    text = path.read_text()
    if canonical:
        for fname, old, new in CANONICAL:
            if path.name == fname:
                if old not in text:
                    raise RuntimeError(f"canonical substitution not found in {path}: {old}")
                text = text.replace(old, new)
    out = []
    for line in text.split("\n"):
        m = re.match(r'\s*#\s*include\s*[<"]([^>"]+)[>"]', line)
        if m:
            name = m.group(1)
            for r in [path.parent] + roots:
                if (r / name).is_file():
                    out.append(_inline_includes(r / name, roots, canonical, seen))
                    break
            else:
                raise RuntimeError(f"include {name} of {path} not found")
            continue
        if re.match(r"\s*#\s*(version|extension)\b", line):
            continue
        out.append(line)
    return "\n".join(out)


def _top_level_statements(text: str):
    """Yields (start, end) of top-level statements (ending in ';' at brace depth 0, or a brace block)."""
    depth = 0
    start = 0
    i = 0
    while i < len(text):
        c = text[i]
        if c == "#" and depth == 0:  # preprocessor line (with its continuation lines)
            j = text.find("\n", i)
            j = len(text) if j < 0 else j
            while text[j - 1] == "\\" and j < len(text):
                j = text.find("\n", j + 1)
                j = len(text) if j < 0 else j
            j = min(j + 1, len(text))
            yield ("pp", start, j)
            i = j
            start = j
            continue
        if c == "{":
            depth += 1
        elif c == "}":
            depth -= 1
            if depth == 0:
                # a function body or a block declaration ends here unless followed by a name / ';'
                k = i + 1
                while k < len(text) and text[k] in " \t\r\n":
                    k += 1
                m = re.match(r"\w*\s*;", text[k:])
                if m:
                    k += m.end()
                    yield ("decl", start, k)
                    i = k
                    start = k
                    continue
                yield ("func", start, i + 1)
                start = i + 1
        elif c == ";" and depth == 0:
            yield ("decl", start, i + 1)
            start = i + 1
        i += 1


def _block_members(body: str):
    for decl in body.split(";"):
        decl = " ".join(decl.split())
        if not decl:
            continue
        yield decl


def _rewrite_decl(stmt: str) -> str:
    s = " ".join(stmt.split())
    if not s or s == ";":
        return stmt
    if re.match(r"layout\s*\(\s*local_size", s):
        return ""
    if s.startswith("struct "):
        return stmt
    # buffer / uniform blocks
    m = re.match(r"((?:layout\s*\([^)]*\)\s*)*)((?:(?:readonly|writeonly|coherent|restrict|volatile)\s+)*)"
                 r"(buffer|uniform)\s+(\w+)\s*\{(.*)\}\s*(\w*)\s*;$", s)
    if m:
        block, body, inst = m.group(4), m.group(5), m.group(6)
        members = []
        for d in _block_members(body):
            am = re.match(r"(.*?)\s*(\w+)\s*\[\s*\]$", d)
            if am:
                members.append(f"glsl::buffer<{am.group(1)}> {am.group(2)};")
            else:
                members.append(d + ";")
        if inst:
            return f"struct {block} {{ {' '.join(members)} }};\nstatic {block} {inst};"
        return "\n".join("static " + x for x in members)
    # opaque uniforms (samplers, images), possibly arrays
    m = re.match(r"((?:layout\s*\([^)]*\)\s*)*)uniform\s+(\w+)\s+(\w+)\s*(\[\s*\])?\s*;$", s)
    if m:
        ty, name = m.group(2), m.group(3)
        if m.group(4):
            return f"static glsl::buffer<glsl::{ty}> {name};"
        return f"static glsl::{ty} {name};"
    m = re.match(r"shared\s+(.*);$", s)
    if m:
        return f"static {m.group(1)};"
    if re.match(r"const\s", s):
        return "static " + s
    # any other global variable is private to an invocation
    if re.match(r"[\w<>]+\s+\w+\s*(\[[^\]]*\])?\s*(=.*)?;$", s):
        return "thread_local " + s
    return stmt


def _rewrite_expressions(text: str) -> str:
    # out / inout parameters
    text = re.sub(r"\b(?:inout|out)\s+(\w+)\s+(\w+)\s*([,)])", r"\1& \2\3", text)
    text = re.sub(r"\bin\s+(\w+)\s+(\w+)\s*([,)])", r"\1 \2\3", text)
    # float literals
    text = re.sub(r"(?<![\w.])(\d+\.\d*(?:[eE][+-]?\d+)?|\.\d+(?:[eE][+-]?\d+)?|\d+[eE][+-]?\d+)(?![\w.])", r"\1f", text)
    # casts
    for ty in ("uint", "int", "float", "bool"):
        text = re.sub(r"(?<![\w.])" + ty + r"\s*\(", f"glsl_{ty}(", text)
    # scalar locals declared without a value (undefined until written in GLSL) start at zero, so that
    # an input that never writes them (a NaN normal in clustered_shading_discretize_normal) is defined
    text = re.sub(r"(?m)^(\s*)(uint|int|float|bool)\s+(\w+)\s*;", r"\1\2 \3 = 0;", text)
    # assignments to swizzles
    def set_swz(m):
        idx = ", ".join(str(SWZ[c]) for c in m.group(2))
        return f"{m.group(1)}.set_swz<{idx}>({m.group(3)});"

    text = re.sub(r"(\b\w+(?:\[[^\]]*\])?)\.([xyzw]{2,3}|[rgb]{2,3})\s*=(?!=)\s*([^;]+);", set_swz, text)
    # swizzles and single components
    def swz(m):
        return ".swz<" + ", ".join(str(SWZ[c]) for c in m.group(1)) + ">()"

    text = re.sub(r"\.([xyzw]{2,4}|[rgba]{2,4})\b(?!\s*[(<])", swz, text)
    text = re.sub(r"\.([rgba])\b(?!\s*[(<\w])", lambda m: "." + "xyzw"[SWZ[m.group(1)]], text)
    text = re.sub(r"\bvoid\s+main\s*\(\s*\)", "void shader_main()", text)
    return text


def _cut_main_for_key(text: str) -> str:
    """find_unique_clusters.comp: keep main() up to the cluster key, return the key."""
    m = re.search(r"void\s+main\s*\(\s*\)\s*\{", text)
    if not m:
        raise RuntimeError("main() not found in find_unique_clusters.comp")
    body_start = m.end()
    cut = text.find("s_cluster_keys[gl_LocalInvocationIndex]", body_start)
    if cut < 0:
        raise RuntimeError("shared-memory store not found in find_unique_clusters.comp")
    prefix = text[body_start:cut]
    return text[: m.start()] + "uint shader_key()\n{" + prefix + "return cluster_key;\n}\n"


def translate(ns: str, rel: str, defines: list[str], keep: str, canonical: bool) -> str:
    ref = reference_dir()
    path = ref / rel
    roots = [ref / "vren/resources/shaders"]
    text = _inline_includes(path, roots, canonical, set())
    if keep == "include":
        text = _inline_includes(roots[0] / "common.glsl", roots, canonical, set()) + "\n" + text
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)  # comments
    text = re.sub(r"//[^\n]*", "", text)
    if keep == "key":
        text = _cut_main_for_key(text)
    pieces = []
    macros = set(defines)
    for kind, a, b in _top_level_statements(text):
        stmt = text[a:b]
        if kind == "pp":
            dm = re.match(r"\s*#\s*define\s+(\w+)", stmt)
            if dm:
                macros.add(dm.group(1))
            pieces.append(stmt)
        elif kind == "decl":
            pieces.append(_rewrite_decl(stmt))
        else:
            pieces.append(stmt)
    body = _rewrite_expressions("".join(pieces))
    head = "".join(f"#define {d}\n" for d in defines)
    tail = "".join(f"#undef {d}\n" for d in sorted(macros))
    return (f"// {rel}\n#undef UINT32_MAX\n{head}namespace {ns} {{\nusing namespace glsl;\n{body}\n}}  // namespace {ns}\n"
            f"{tail}")


def generate(variant: str) -> str:
    canonical = variant == "canonical"
    parts = [f"// Generated by oracle/ref_shaders.py ({variant} variant) from the reference's shader sources.\n"]
    for ns, rel, defines, keep in SHADERS:
        parts.append(translate(ns, rel, defines, keep, canonical))
    return "\n".join(parts)


def build(verbose: bool = False) -> dict | None:
    """Generates and compiles both variants; returns {variant: library path}, or None when the
    reference checkout is absent (the libraries already built, if any, stay usable)."""
    ref = reference_dir()
    if not (ref / "vren/resources/shaders").is_dir():
        return None
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        raise RuntimeError("g++ is required to build oracle/_ref")
    OUT_DIR.mkdir(exist_ok=True)
    libs = {}
    for variant in VARIANTS:
        gen = OUT_DIR / f"ref_shaders_{variant}.inc"
        text = generate(variant)
        if not gen.exists() or gen.read_text() != text:
            gen.write_text(text)
        lib = OUT_DIR / f"libvren_ref_{variant}.so"
        deps = [gen, DRIVERS, HEADER]
        if not lib.exists() or any(d.stat().st_mtime > lib.stat().st_mtime for d in deps):
            tmp = lib.with_suffix(".so.tmp")
            cmd = [cxx, "-std=c++20", "-O2", "-fPIC", "-shared", "-pthread", "-ffp-contract=off", "-fno-fast-math",
                   "-w", f"-I{ORACLE_DIR}", f"-I{OUT_DIR}", f'-DVREN_REF_INC="ref_shaders_{variant}.inc"',
                   f"-DVREN_REF_CANONICAL={1 if variant == 'canonical' else 0}", str(DRIVERS), "-o", str(tmp)]
            if verbose:
                print(" ".join(cmd))
            subprocess.run(cmd, check=True)
            os.replace(tmp, lib)
        libs[variant] = lib
    return libs


if __name__ == "__main__":
    print(build(verbose=True))
