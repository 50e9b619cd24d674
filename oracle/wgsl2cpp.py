"""Mechanical WGSL -> C++ translation of the reference's compute shaders.

Test infrastructure only.  The reference (PPLUSCHT/LBM, crate lbm-wgpu) keeps
its whole numerical path in WGSL compute shaders; it has no CPU path and no
tests, and no graphics or compute API is available here.  This script turns
the WGSL files (read where they lie in the reference tree) into one C++ header
that oracle/ref_host.cpp drives in the reference's dispatch order, so the CPU
oracle restatement can be checked against the reference's own shader code.

Only the WGSL subset these shaders use is handled: struct declarations,
storage / uniform bindings, helper functions, one @compute entry point,
`let`, `if`/`else`, `switch` on an integer with braced cases, `return`,
compound assignment, f32/u32 literals, vec3 values (construction, scalar
products, sums) and the built-ins clamp, sqrt, floor and i32().  Semantics
kept:
  * f32 literals become C++ float literals (f32 arithmetic, no promotion);
  * u32 arithmetic wraps (uint32_t);
  * runtime-sized array reads and writes clamp the index to the last element
    (naga's "Restrict" bounds-check policy);
  * no FMA contraction (the generated code is compiled with -ffp-contract=off);
  * a WGSL case never falls through (each translated case ends in `break`);
  * `1 - x` with an abstract integer and an f32 is f32 arithmetic.
Anything outside the subset raises, so a shader change cannot slip through
silently.

Usage: python wgsl2cpp.py OUT.inc NAME=path/to/shader.wgsl [NAME=...]
"""
import re
import sys

TYPE_MAP = {"f32": "float", "u32": "uint32_t", "i32": "int32_t", "vec3<u32>": "uvec3", "vec3<f32>": "vec3f"}

PRELUDE = """// Generated by oracle/wgsl2cpp.py from the reference's WGSL shaders. Do not edit.
#pragma once
#include <cstdint>
#include <cmath>
namespace wgsl {
struct uvec3 { uint32_t x, y, z; };
template <class T> struct RArr {
  T* p = nullptr; uint32_t n = 0;
  T& operator[](uint32_t i) const { return p[i < n ? i : n - 1]; }
};
static inline float clamp(float e, float lo, float hi) { return std::fmin(std::fmax(e, lo), hi); }
static inline float sqrt(float v) { return std::sqrt(v); }
static inline float floor(float v) { return std::floor(v); }
static inline int32_t i32(float v) { return (int32_t)v; }
struct vec3f { float x, y, z; };
static inline vec3f vec3(float x, float y, float z) { return vec3f{x, y, z}; }
static inline vec3f operator*(float a, vec3f v) { return vec3f{a * v.x, a * v.y, a * v.z}; }
static inline vec3f operator+(vec3f a, vec3f b) { return vec3f{a.x + b.x, a.y + b.y, a.z + b.z}; }
}  // namespace wgsl
"""


def ctype(t):
    t = t.strip()
    if t in TYPE_MAP:
        return TYPE_MAP[t]
    if re.fullmatch(r"[A-Za-z_]\w*", t):
        return t
    raise ValueError("unsupported WGSL type: %r" % t)


def strip_comments(src):
    return re.sub(r"//[^\n]*", "", src)


def _block_end(src, i):
    """Index just past the brace block that opens at src[i] == '{'."""
    depth = 0
    for j in range(i, len(src)):
        if src[j] == "{":
            depth += 1
        elif src[j] == "}":
            depth -= 1
            if depth == 0:
                return j + 1
    raise ValueError("unbalanced braces")


def translate_switches(src):
    """`switch e { case k: {..} default: {..} }` -> C++ with a break after
    every case block (WGSL cases do not fall through)."""
    out, pos = [], 0
    for m in re.finditer(r"\bswitch\s+([^{]+?)\s*\{", src):
        if m.start() < pos:
            raise ValueError("nested switch")
        out.append(src[pos:m.start()])
        end = _block_end(src, m.end() - 1)
        body = src[m.end():end - 1]
        parts, bpos = [], 0
        for c in re.finditer(r"(case\s+-?\d+|default)\s*:\s*\{", body):
            if c.start() < bpos:
                continue
            cend = _block_end(body, c.end() - 1)
            if body[bpos:c.start()].strip():
                raise ValueError("unsupported switch body")
            parts.append("%s: %s break;" % (c.group(1), body[c.end() - 1:cend]))
            bpos = cend
        if body[bpos:].strip():
            raise ValueError("unsupported switch body")
        out.append("switch (%s) {\n%s\n}" % (m.group(1).strip(), "\n".join(parts)))
        pos = end
    out.append(src[pos:])
    return "".join(out)


def translate(name, src):
    src = strip_comments(src)
    out = ["namespace %s {" % name, "using namespace wgsl;"]
    pos = 0
    fn_names = re.findall(r"\bfn\s+([A-Za-z_]\w*)\s*\(", src)
    helpers = [f for f in fn_names if f != "main"]
    body_chunks = []

    # struct declarations
    for m in re.finditer(r"struct\s+(\w+)\s*\{([^}]*)\}", src):
        fields = []
        for fld in m.group(2).split(","):
            fld = fld.strip()
            if not fld:
                continue
            fname, ftype = [s.strip() for s in fld.split(":")]
            fields.append("  %s %s;" % (ctype(ftype), fname))
        out.append("struct %s {\n%s\n};" % (m.group(1), "\n".join(fields)))
    src_nostruct = re.sub(r"struct\s+(\w+)\s*\{([^}]*)\}", "", src)

    # bindings
    for m in re.finditer(r"@group\(\d+\)\s*@binding\(\d+\)\s*var<([^>]*)>\s*(\w+)\s*:\s*([^;]+);",
                         src_nostruct):
        space, vname, vtype = m.group(1), m.group(2), m.group(3).strip()
        am = re.fullmatch(r"array<\s*(.+?)\s*>", vtype)
        if am:
            out.append("RArr<%s> %s;" % (ctype(am.group(1)), vname))
        elif space.strip() == "uniform":
            out.append("%s %s{};" % (ctype(vtype), vname))
        else:
            raise ValueError("unsupported binding %r" % m.group(0))
    rest = re.sub(r"@group\(\d+\)\s*@binding\(\d+\)\s*var<[^>]*>\s*\w+\s*:\s*[^;]+;", "", src_nostruct)
    rest = re.sub(r"@compute|@workgroup_size\([^)]*\)|@builtin\(\w+\)", "", rest)

    # functions
    def params(p):
        res = []
        for item in [s.strip() for s in p.split(",") if s.strip()]:
            item = re.sub(r"@builtin\(\w+\)\s*", "", item)
            pn, pt = [s.strip() for s in item.split(":", 1)]
            res.append("%s %s" % (ctype(pt), pn))
        return ", ".join(res)

    def fn_header(m):
        fname, p, ret = m.group(1), m.group(2), m.group(3)
        cret = ctype(ret) if ret else "void"
        cname = "entry" if fname == "main" else "fn_" + fname
        return "static inline %s %s(%s)" % (cret, cname, params(p))

    rest = re.sub(r"\bfn\s+(\w+)\s*\(([^)]*)\)\s*(?:->\s*([\w<>]+))?\s*", lambda m: fn_header(m) + " ", rest)
    # statements
    rest = re.sub(r"\blet\s+(\w+)\s*=", r"const auto \1 =", rest)
    if re.search(r"\bvar\b|\bloop\b|\bfor\b|\bwhile\b|\bvec[24]|\bvec3<|\bselect\(|\bfallthrough\b", rest):
        raise ValueError("WGSL construct outside the supported subset in %s" % name)
    rest = translate_switches(rest)
    # f32 literals (not inside identifiers), then helper-function calls
    rest = re.sub(r"(?<![\w.])(\d+\.\d*)(?![\w.])", r"\1f", rest)
    for h in helpers:
        rest = re.sub(r"(?<![\w.])%s\s*\(" % re.escape(h), "fn_%s(" % h, rest)
    out.append(rest.strip())
    out.append("}  // namespace %s" % name)
    return "\n".join(out)


def main(argv):
    if len(argv) < 3:
        print(__doc__)
        return 2
    out_path = argv[1]
    parts = [PRELUDE]
    for spec in argv[2:]:
        name, path = spec.split("=", 1)
        with open(path) as f:
            parts.append("// from %s\n" % path.split("lbm-wgpu/", 1)[-1] + translate(name, f.read()))
    with open(out_path, "w") as f:
        f.write("\n\n".join(parts) + "\n")
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv))
