"""Compiles the reference's own GLSL compute shaders as host C++.

TEST INFRASTRUCTURE ONLY.  This recipe reads the reference's shader sources
where they lie (`RaytracerGPU_MastersProject/shaders/compute/*.comp` and
`shaders/include/*.glsl` under the reference checkout, default
/root/reference, or $RT_REFERENCE_ROOT), rewrites the GLSL-only syntax around
them into C++ and compiles them, with oracle/ref_shim.hpp (GLSL types and
built-ins) and oracle/ref_harness.cpp (dispatch entry points), into
oracle/_ref/libref_glsl.so (sin/cos from libm) and
oracle/_ref/libref_glsl_portable.so (the oracle's portable sin/cos).  The
generated sources and libraries stay in oracle/_ref/, which is not committed.
On a host without the reference checkout, previously generated sources in
oracle/_ref/ are compiled again; with neither, nothing is built.

The rewrite changes syntax only, never an expression:
  * `#include "..."` is inlined, `#version` / `#extension` lines dropped,
    comments blanked (line numbers kept, `#line` directives point back at the
    shader file);
  * the shader becomes the body of a class deriving glsl::InvocationBase:
    its globals become members whose initialisers run per invocation, as a
    GLSL global initialiser does, and its functions member functions;
  * `layout(binding = N) uniform|buffer Block { ... } inst;` becomes a
    reference member bound to descriptor N; an anonymous block holding one
    runtime-sized array `T name[ ];` becomes a pointer member `T* name`
    (`const T*` when the block is readonly); `uniform image2D x` a reference
    to the bound image; `layout(local_size_x = X ...) in;` the constants
    kLocalSizeX/Y/Z;
  * `shared uint x` / `shared uint[N] x` become static atomic words
    (`shared T[N] x` becomes a static `T x[N]` for other T);
  * parameter qualifiers: `in T x` -> `T x`, `out/inout T x` -> `T& x`;
  * floating literals without a suffix get `f` (GLSL literals are binary32);
  * `uint(expr)` becomes glsl_uint(expr) (saturating from float) and a
    scalar `.xxx` swizzle glsl_xxx(...).
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
REF_SUBDIR = "RaytracerGPU_MastersProject"

# kernel name -> shader file, relative to RaytracerGPU_MastersProject/
KERNELS = {
    "raytraceBVH": "shaders/compute/raytraceBVH.comp",
    "ModelSpaceToWorldSpace": "shaders/compute/ModelSpaceToWorldSpace.comp",
    "GetEnclosingAABB": "shaders/compute/GetEnclosingAABB.comp",
    "GenerateMortonCodesOfPrimitives": "shaders/compute/GenerateMortonCodesOfPrimitives.comp",
    "RadixSortSimple": "shaders/compute/RadixSortSimple.comp",
    "ConstructHLBVH": "shaders/compute/ConstructHLBVH.comp",
    "ConstructAABBsOfInternalNodes": "shaders/compute/ConstructAABBsOfInternalNodes.comp",
}

LIBS = {"libref_glsl.so": [], "libref_glsl_portable.so": ["-DREF_PORTABLE_SINCOS"]}


def reference_root() -> Path | None:
    root = Path(os.environ.get("RT_REFERENCE_ROOT", "/root/reference")) / REF_SUBDIR
    return root if (root / KERNELS["raytraceBVH"]).exists() else None


# ----------------------------------------------------------------- rewrite --
def _blank_comments(text: str) -> str:
    def keep_newlines(m: re.Match) -> str:
        return re.sub(r"[^\n]", " ", m.group(0))

    return re.sub(r"//[^\n]*|/\*.*?\*/", keep_newlines, text, flags=re.S)


def _inline(path: Path, rel: str) -> str:
    """Shader text with its includes inlined, each file's lines under a #line."""
    out = [f'#line 1 "{rel}"']
    for i, line in enumerate(path.read_text().splitlines(), 1):
        m = re.match(r'\s*#\s*include\s+"([^"]+)"', line)
        if m:
            inc = (path.parent / m.group(1)).resolve()
            inc_rel = str(Path(rel).parent / m.group(1))
            out.append(_inline(inc, os.path.normpath(inc_rel)))
            out.append(f'#line {i + 1} "{rel}"')
        elif re.match(r"\s*#\s*(version|extension)\b", line):
            out.append("")
        else:
            out.append(line)
    return "\n".join(out)


def _binding(layout: str) -> int:
    m = re.search(r"binding\s*=\s*(\d+)", layout)
    if not m:
        raise ValueError(f"no binding in layout({layout})")
    return int(m.group(1))


def _nl(s: str) -> str:
    """The newlines of a replaced span, so that line numbers stay."""
    return "\n" * s.count("\n")


def translate(text: str) -> tuple[str, list[str]]:
    """-> (class body, macro names the shader defines)."""
    text = _blank_comments(text)
    macros = re.findall(r"^\s*#\s*define\s+(\w+)", text, flags=re.M)

    # layout(local_size_x = X, ...) in;
    def local_size(m: re.Match) -> str:
        args = dict(re.findall(r"local_size_([xyz])\s*=\s*([^,)]+)", m.group(1)))
        dims = [args.get(k, "1").strip() for k in "xyz"]
        return (f"static constexpr uint kLocalSizeX = {dims[0]}, kLocalSizeY = {dims[1]}, "
                f"kLocalSizeZ = {dims[2]};" + _nl(m.group(0)))

    text = re.sub(r"layout\s*\(([^)]*local_size[^)]*)\)\s*in\s*;", local_size, text)

    # uniform / buffer blocks
    def block(m: re.Match) -> str:
        layout, quals, kind, name, body, inst = m.groups()
        n = _binding(layout)
        readonly = "readonly" in (quals or "")
        if inst:
            return f"struct {name} {{{body}}}; {name}& {inst} = *static_cast<{name}*>(env.bind[{n}]);"
        arr = re.fullmatch(r"\s*(\w+)\s+(\w+)\s*\[\s*\]\s*;\s*", body)
        if not arr:
            raise ValueError(f"block {name}: expected one runtime-sized array")
        t, var = arr.groups()
        c = "const " if readonly else ""
        return f"{c}{t}* {var} = static_cast<{c}{t}*>(env.bind[{n}]);" + _nl(m.group(0))

    text = re.sub(r"layout\s*\(([^)]*)\)\s*((?:(?:readonly|writeonly|coherent|restrict|volatile)\s+)*)"
                  r"(uniform|buffer)\s+(\w+)\s*\{([^}]*)\}\s*(\w*)\s*;", block, text)

    # uniform image2D x;
    def image(m: re.Match) -> str:
        return f"image2D& {m.group(3)} = *static_cast<image2D*>(env.bind[{_binding(m.group(1))}]);"

    text = re.sub(r"layout\s*\(([^)]*)\)\s*((?:(?:readonly|writeonly|coherent)\s+)*)uniform\s+image2D\s+(\w+)\s*;",
                  image, text)

    # shared declarations
    def shared(m: re.Match) -> str:
        t, dim, var = m.group(1), m.group(2), m.group(3)
        t = "::glsl::shared_u32" if t == "uint" else t
        suffix = f"[{dim.strip()[1:-1]}]" if dim else ""
        return f"static inline {t} {var}{suffix};"

    text = re.sub(r"^\s*shared\s+(\w+)\s*(\[[^\]]*\])?\s+(\w+)\s*;", shared, text, flags=re.M)

    # parameter qualifiers of function definitions (column-0 signatures)
    def params(m: re.Match) -> str:
        p = m.group(3)
        p = re.sub(r"\b(?:inout|out)\s+(\w+)\s+(\w+)", r"\1& \2", p)
        p = re.sub(r"\bin\s+(\w+)\s+(\w+)", r"\1 \2", p)
        return f"{m.group(1)} {m.group(2)}({p}){m.group(4)}"

    text = re.sub(r"^(\w+)\s+(\w+)\s*\(([^()]*)\)(\s*\{)", params, text, flags=re.M)

    # binary32 literals
    text = re.sub(r"(?<![\w.])(\d+\.\d*|\.\d+)([eE][+-]?\d+)?(?![\w.])", r"\1\2f", text)
    # conversions and scalar swizzles
    text = re.sub(r"(?<![\w.])uint\s*\(", "glsl_uint(", text)
    text = re.sub(r"([\w.\[\]]+)\.xxx\b", r"glsl_xxx(\1)", text)
    return text, sorted(set(macros))


def generate(root: Path) -> None:
    OUT.mkdir(exist_ok=True)
    for name, rel in KERNELS.items():
        body, macros = translate(_inline(root / rel, rel))
        undefs = "\n".join(f"#undef {m}" for m in macros)
        src = (f"// Generated by oracle/ref_glsl.py from {REF_SUBDIR}/{rel}: the shader's text as a\n"
               f"// C++ class (see ref_glsl.py for the syntax rewrites).  Not committed.\n"
               f"namespace glsl {{\nnamespace k_{name} {{\n"
               f"struct Invocation : InvocationBase {{\n  using InvocationBase::InvocationBase;\n"
               f"{body}\n#line 1 \"k_{name}.inc\"\n}};\n}}  // namespace k_{name}\n}}  // namespace glsl\n{undefs}\n")
        path = OUT / f"k_{name}.inc"
        if not path.exists() or path.read_text() != src:
            path.write_text(src)


def compile_libs() -> list[Path]:
    srcs = [HERE / "ref_harness.cpp", HERE / "ref_shim.hpp", HERE / "rt_sincos.h"] + sorted(OUT.glob("k_*.inc"))
    newest = max(p.stat().st_mtime for p in srcs)
    cxx = os.environ.get("CXX", "g++")

    def one(item):
        lib, defs = item
        out = OUT / lib
        if out.exists() and out.stat().st_mtime >= newest:
            return out
        tmp = out.with_suffix(".so.tmp")
        cmd = [cxx, "-std=c++20", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-pthread",
               "-w", *defs, f"-I{HERE}", f"-I{OUT}", "-o", str(tmp), str(HERE / "ref_harness.cpp")]
        subprocess.run(cmd, check=True, capture_output=True, text=True)
        tmp.replace(out)
        return out

    with ThreadPoolExecutor(len(LIBS)) as ex:
        return list(ex.map(one, LIBS.items()))


def build() -> list[Path]:
    """Generates (when the reference checkout is present) and compiles the
    libraries; returns their paths, or [] when neither the reference nor
    previously generated sources exist."""
    root = reference_root()
    if root is not None:
        generate(root)
    if not all((OUT / f"k_{k}.inc").exists() for k in KERNELS):
        return []
    return compile_libs()


if __name__ == "__main__":
    try:
        built = build()
    except subprocess.CalledProcessError as e:
        sys.stderr.write(e.stderr or "")
        raise
    print("\n".join(str(p) for p in built) if built else "reference shaders not found: nothing built")
