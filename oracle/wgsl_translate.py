#!/usr/bin/env python3
"""TEST INFRASTRUCTURE ONLY: build the reference's own simulation shaders as C++.

Reads the reference's TypeScript sources in place (src/engine/wgsl.ts,
src/engine/f1.ts, src/engine/car-model.ts), extracts the WGSL template strings
of the four simulation modules that the engine dispatches
(LBM_INIT wgsl.ts:141, LBM_STEP wgsl.ts:157, VOXELIZE wgsl.ts:294,
HEAT wgsl.ts:460, with every chunk they concatenate: GRID, SHAPE, D3Q19,
SDF_PRIMITIVES, SDF_F1, RIG_WGSL, SDF_SCENE), and rewrites the WGSL syntax into
C++ that compiles against oracle/wgsl_runtime.hpp.  Only syntax changes; the
arithmetic, branch order and constants stay those of the shader text.

Output goes to oracle/_ref/ only (git-ignored):
    oracle/_ref/wgsl_modules.inc   translated modules, one C++ namespace each
The Makefile then compiles oracle/ref_driver.cpp (which emulates the WebGPU
dispatches of src/engine/engine.ts) into oracle/_ref/libwgslref.so.

WGSL semantics carried over explicitly:
  * float literals become f32 literals; a product or quotient of two literals
    (an AbstractFloat expression, e.g. `18.0 * 1.41421356` at wgsl.ts:261) is
    evaluated in double and rounded once to f32, as WGSL constant evaluation does;
  * i32(), u32(), f32() conversions map to saturating runtime conversions;
  * compute entry points are split at top-level workgroupBarrier() into phases
    that the driver runs for every invocation of a workgroup in turn;
  * var<private>/var<workgroup> become thread_local, so workgroups can run on
    several host threads.
"""
import os
import re
import struct
import sys

REF = os.environ.get("WT_REFERENCE_ROOT", "/root/reference")
HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")


# ---------------------------------------------------------------- TS extraction
def _template_literal(src, i):
    """src[i] == '`'; return (text, index after closing backtick)."""
    assert src[i] == "`"
    i += 1
    out = []
    while src[i] != "`":
        if src[i] == "$" and src[i + 1] == "{":
            depth, j = 1, i + 2
            while depth:
                depth += {"{": 1, "}": -1}.get(src[j], 0)
                j += 1
            out.append(("expr", src[i + 2 : j - 1]))
            i = j
        else:
            j = i
            while src[j] != "`" and not (src[j] == "$" and src[j + 1] == "{"):
                j += 1
            out.append(("text", src[i:j]))
            i = j
    return out, i + 1


def extract_consts(path):
    """Map NAME -> list of parts ('ident', name) | ('tmpl', parts) for `const NAME = a + `..` + b;`."""
    src = open(path).read()
    res = {}
    for m in re.finditer(r"(?:export\s+)?const\s+([A-Z0-9_]+)\s*=\s*", src):
        name, i = m.group(1), m.end()
        parts = []
        while True:
            while src[i] in " \n\t":
                i += 1
            if src.startswith("/*", i):
                i = src.index("*/", i) + 2
                continue
            if src[i] == "`":
                t, i = _template_literal(src, i)
                parts.append(("tmpl", t))
            else:
                mm = re.match(r"[A-Za-z_][A-Za-z0-9_]*", src[i:])
                if not mm:
                    break
                parts.append(("ident", mm.group(0)))
                i += len(mm.group(0))
            while src[i] in " \n\t":
                i += 1
            if src[i] == "+":
                i += 1
                continue
            break
        if parts and any(p[0] == "tmpl" for p in parts) or (parts and all(p[0] == "ident" for p in parts) and src[i] == ";"):
            res[name] = parts
    return res


def rig_constants(path):
    """Numbers interpolated into RIG_WGSL (car-model.ts:40-50 RIG object)."""
    src = open(path).read()
    m = re.search(r"export const RIG = \{(.*?)\n\};", src, re.S)
    body = m.group(1)
    front = re.search(r"front:\s*\{(.*?)\}", body).group(1)
    vals = {
        "RIG.front.fadeIn[0]": re.search(r"fadeIn:\s*\[([-\d.]+)", front).group(1),
        "RIG.front.fadeIn[1]": re.search(r"fadeIn:\s*\[[-\d.]+,\s*([-\d.]+)", front).group(1),
        "RIG.front.fadeOut[0]": re.search(r"fadeOut:\s*\[([-\d.]+)", front).group(1),
        "RIG.front.fadeOut[1]": re.search(r"fadeOut:\s*\[[-\d.]+,\s*([-\d.]+)", front).group(1),
        "RIG.front.dz": re.search(r"dz:\s*([-\d.]+)", front).group(1),
        "RIG.front.bins - 1": str(int(re.search(r"bins:\s*(\d+)", front).group(1)) - 1),
        "RIG.frontThinFactor": re.search(r"frontThinFactor:\s*([-\d.]+)", body).group(1),
    }
    return vals


def resolve(name, table, rig, seen=()):
    parts = table[name]
    out = []
    for kind, v in parts:
        if kind == "ident":
            out.append(resolve(v, table, rig, seen + (name,)))
        else:
            for k, t in v:
                if k == "text":
                    out.append(t)
                else:
                    key = t.strip()
                    if key not in rig:
                        raise SystemExit(f"unknown template expression ${{{key}}} in {name}")
                    out.append(rig[key])
    return "".join(out)


# ---------------------------------------------------------------- WGSL -> C++
FLOAT_RE = r"(?:\d+\.\d*(?:[eE][-+]?\d+)?|\.\d+(?:[eE][-+]?\d+)?|\d+[eE][-+]?\d+)"


def f32_literal(x):
    f = struct.unpack("<f", struct.pack("<f", x))[0]
    return float(f).hex() + "f"


def fold_abstract(code, report):
    # AbstractFloat products/quotients of two literals: evaluate in double, round once.
    pat = re.compile(r"(?P<pre>[=(,+\-]\s*)(?P<a>" + FLOAT_RE + r")\s*(?P<op>[*/])\s*(?P<b>" + FLOAT_RE + r")(?![\w.])")

    def rep(m):
        a, b = float(m.group("a")), float(m.group("b"))
        v = a * b if m.group("op") == "*" else a / b
        report.append(f"{m.group('a')} {m.group('op')} {m.group('b')} -> {v!r}")
        return m.group("pre") + f32_literal(v)

    return pat.sub(rep, code)


def suffix_floats(code):
    pat = re.compile(r"(?<![\w.])(" + FLOAT_RE + r")(?![\w.])")
    return pat.sub(lambda m: m.group(1) + "f", code)


def split_top(s, sep=","):
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch in "<([":
            depth += 1
        elif ch in ">)]":
            depth -= 1
        if ch == sep and depth == 0:
            out.append(cur)
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur)
    return out


def read_type(s, i):
    """Parse a WGSL type starting at s[i]; return (type, end)."""
    m = re.match(r"\s*([A-Za-z_][A-Za-z0-9_]*)", s[i:])
    t = m.group(1)
    j = i + m.end()
    if j < len(s) and s[j] == "<":
        depth, k = 0, j
        while True:
            depth += {"<": 1, ">": -1}.get(s[k], 0)
            k += 1
            if depth == 0:
                break
        t += s[j:k]
        j = k
    return t, j


def cxx_type(t):
    t = t.strip()
    m = re.match(r"array<(.*)>$", t)
    if m:
        parts = split_top(m.group(1))
        if len(parts) == 1:
            return None  # runtime-sized: only valid for storage bindings
        return f"array<{cxx_type(parts[0])}, {parts[1].strip().rstrip('u')}>"
    m = re.match(r"atomic<(.*)>$", t)
    if m:
        return f"atomic<{cxx_type(m.group(1))}>"
    m = re.match(r"ptr<\s*function\s*,\s*(.*)>$", t)
    if m:
        return f"{cxx_type(m.group(1))}*"
    if t == "texture_3d<f32>":
        return "texture3d"
    if t == "texture_2d<f32>":
        return "texture2d"
    if t == "sampler":
        return "sampler"
    return t


def storage_elem(t):
    m = re.match(r"array<(.*)>$", t.strip())
    parts = split_top(m.group(1))
    return cxx_type(parts[0])


CXX_KEYWORDS = {"default_", "new", "delete", "this", "union", "char", "short", "long", "double", "int",
                "float", "signed", "unsigned", "register", "auto", "template", "typename", "class",
                "private", "public", "protected", "operator", "namespace", "using", "friend", "virtual"}


def translate_module(name, wgsl, report):
    code = wgsl
    code = re.sub(r"@compute\s*@workgroup_size\([^)]*\)\s*", "", code)
    code = fold_abstract(code, report)
    code = suffix_floats(code)
    code = re.sub(r"\b(i32|u32|f32)\(", r"to_\1(", code)
    code = re.sub(r"\.([xyzw]{2,4}|[rgba]{2,4})\b", swizzle, code)
    code = re.sub(r"\.([rgba])\b", lambda m: "." + "xyzw"["rgba".index(m.group(1))], code)
    # render-pipeline entry points become plain functions the driver calls per
    # pixel / per vertex; interface attributes carry no arithmetic
    code = re.sub(r"@(fragment|vertex)\s*", "", code)
    code = re.sub(r"@location\(\d+\)\s*", "", code)
    code = re.sub(r"@interpolate\([^)]*\)\s*", "", code)
    struct_names = re.findall(r"\bstruct\s+(\w+)", code)

    structs, globs, protos, funcs = [], [], [], []
    entry = None
    i = 0
    # WGSL module-scope declarations are order independent; C++ needs structs,
    # then globals, then prototypes, then function bodies.
    while i < len(code):
        m = re.match(r"\s+", code[i:])
        if m:
            i += m.end()
            continue
        if code.startswith("//", i):
            i = code.index("\n", i)
            continue
        if code.startswith("struct", i):
            m = re.match(r"struct\s+(\w+)\s*\{", code[i:])
            j = code.index("}", i)
            body = code[i + m.end() : j]
            fields = []
            for ln in body.split("\n"):
                ln = re.sub(r"//.*", "", ln)
                ln = re.sub(r"@builtin\(\w+\)\s*", "", ln)
                for f in split_top(ln):
                    if ":" in f:
                        fn, ft = f.split(":", 1)
                        fields.append(f"  {cxx_type(ft)} {fn.strip()};")
            structs.append(f"struct {m.group(1)} {{\n" + "\n".join(fields) + "\n};")
            i = j + 1
            continue
        m = re.match(r"@group\(\d+\)\s*@binding\(\d+\)\s*var(<[^>]*>)?\s+(\w+)\s*:\s*", code[i:])
        if m:
            space, vname = (m.group(1) or ""), m.group(2)
            t, j = read_type(code, i + m.end())
            j = code.index(";", j) + 1
            if "storage" in space:
                globs.append(f"inline storage<{storage_elem(t)}> {vname};")
            else:
                globs.append(f"inline {cxx_type(t)} {vname}{{}};")
            i = j
            continue
        m = re.match(r"var<(private|workgroup)>\s+(\w+)\s*:\s*", code[i:])
        if m:
            t, j = read_type(code, i + m.end())
            j = code.index(";", j) + 1
            globs.append(f"static thread_local {cxx_type(t)} {m.group(2)}{{}};")
            i = j
            continue
        m = re.match(r"const\s+(\w+)\s*(:\s*)?", code[i:])
        if m:
            if m.group(2):
                t, j = read_type(code, i + m.end())
                ctype = cxx_type(t)
            else:
                ctype, j = "auto", i + m.end()
            k = code.index(";", j)
            init = code[j:k].strip().lstrip("=").strip()
            globs.append(f"static const {ctype} {m.group(1)} = {stmt_rewrite(init)};")
            i = k + 1
            continue
        m = re.match(r"fn\s+(\w+)\s*\(", code[i:])
        if m:
            fname = m.group(1)
            depth, j = 1, i + m.end()
            while depth:
                depth += {"(": 1, ")": -1}.get(code[j], 0)
                j += 1
            params_src = code[i + m.end() : j - 1]
            mm = re.match(r"\s*->\s*", code[j:])
            ret = "void"
            if mm:
                ret, j = read_type(code, j + mm.end())
                ret = cxx_type(ret)
            b0 = code.index("{", j)
            depth, k = 1, b0 + 1
            while depth:
                depth += {"{": 1, "}": -1}.get(code[k], 0)
                k += 1
            body = code[b0 + 1 : k - 1]
            params, builtins = [], []
            for p in split_top(params_src):
                p = p.strip()
                if not p:
                    continue
                bm = re.match(r"@builtin\((\w+)\)\s*", p)
                if bm:
                    builtins.append(bm.group(1))
                    p = p[bm.end() :]
                pn, pt = p.split(":", 1)
                params.append(f"{cxx_type(pt)} {pn.strip()}")
            if fname == "cs_main":
                entry = (params, builtins, body)
            else:
                sig = f"static {ret} {fname}({', '.join(params)})"
                protos.append(sig + ";")
                body = brace_structs(ordered_constructors(body), struct_names)
                body = re.sub(r"\bdiscard\s*;", "{ rt_discarded = true; return {}; }", body)
                funcs.append(sig + " {" + stmt_rewrite(body) + "}")
            i = k
            continue
        raise SystemExit(f"{name}: cannot parse near: {code[i:i+80]!r}")

    if "rt_discarded" in "".join(funcs):
        globs.append("static thread_local bool rt_discarded = false;")
    if entry is None:  # render module: fs_main / vs_main are called directly
        return "\n".join([f"namespace {name} {{", "RT_USING", *structs, *globs, *protos, *funcs,
                          f"}}  // namespace {name}", ""])
    params, builtins, body = entry
    phases = re.split(r"\bworkgroupBarrier\(\)\s*;", body)
    ent = []
    for pi, ph in enumerate(phases):
        ent.append(f"static void cs_main_phase{pi}({', '.join(params)}) {{{stmt_rewrite(ph)}}}")
    args = [{"global_invocation_id": "gid", "local_invocation_index": "li"}[b] for b in builtins]
    ent.append(f"static const int cs_main_nphases = {len(phases)};")
    ent.append("static inline void cs_main_run(int phase, vec3u gid, u32 li) {")
    ent.append("  (void)gid; (void)li;")
    ent.append("  switch (phase) {")
    for pi in range(len(phases)):
        ent.append(f"    case {pi}: cs_main_phase{pi}({', '.join(args)}); break;")
    ent.append("  }")
    ent.append("}")
    return "\n".join([f"namespace {name} {{", "RT_USING", *structs, *globs, *protos, *funcs, *ent,
                      f"}}  // namespace {name}", ""])


def swizzle(m):
    """v.xzy / v.rgb -> v.swz<0,2,1>() (a member template of the runtime's vectors)."""
    letters = m.group(1)
    names = "xyzw" if letters[0] in "xyzw" else "rgba"
    return ".swz<" + ",".join(str(names.index(c)) for c in letters) + ">()"


def brace_structs(s, names):
    """Struct constructors Name(a, b, ...) -> Name{a, b, ...}: aggregate
    initialisation, whose initialisers C++ evaluates left to right as WGSL does."""
    if not names:
        return s
    out, i = [], 0
    for m in re.finditer(r"\b(" + "|".join(names) + r")\(", s):
        if m.start() < i:
            continue
        depth, j = 1, m.end()
        while depth:
            depth += {"(": 1, ")": -1}.get(s[j], 0)
            j += 1
        out.append(s[i:m.start()] + m.group(1) + "{" + brace_structs(s[m.end():j - 1], names) + "}")
        i = j
    out.append(s[i:])
    return "".join(out)


def ordered_constructors(s):
    """WGSL evaluates call arguments left to right; C++ leaves the order open.
    Vector constructors whose arguments call rand() (which advances the seed it
    points to) become braced initialisers, which C++ evaluates in order."""
    out, i = [], 0
    for m in re.finditer(r"\bvec[234][fiu]\(", s):
        if m.start() < i:
            continue
        depth, j = 1, m.end()
        while depth:
            depth += {"(": 1, ")": -1}.get(s[j], 0)
            j += 1
        args = s[m.end():j - 1]
        if "rand(" in args:
            out.append(s[i:m.start()] + s[m.start():m.end() - 1] + "{" + ordered_constructors(args) + "}")
            i = j
    out.append(s[i:])
    return "".join(out)


def stmt_rewrite(s):
    """let/var declarations -> C++ declarations (WGSL var is zero-initialised)."""
    out = []
    i = 0
    while i < len(s):
        m = re.match(r"(let|var)\s+(\w+)\s*", s[i:])
        if m and (i == 0 or not (s[i - 1].isalnum() or s[i - 1] in "_.")):
            kind, nm = m.group(1), m.group(2)
            j = i + m.end()
            if s[j] == ":":
                t, j = read_type(s, j + 1)
                ct = cxx_type(t)
                k = j
                while s[k] in " \t":
                    k += 1
                if s[k] == ";":
                    out.append(f"{ct} {nm}{{}}")
                    i = k
                    continue
                out.append(("const " if kind == "let" else "") + f"{ct} {nm} ")
                i = j
                continue
            out.append(("const auto " if kind == "let" else "auto ") + f"{nm} ")
            i = j
            continue
        out.append(s[i])
        i += 1
    return "".join(out)


def main():
    eng = os.path.join(REF, "src", "engine")
    table = {}
    for f in ("wgsl.ts", "f1.ts", "car-model.ts", "render-wgsl.ts"):
        table.update(extract_consts(os.path.join(eng, f)))
    rig = rig_constants(os.path.join(eng, "car-model.ts"))
    report = []
    mods = {
        "m_lbm_init": "LBM_INIT",
        "m_lbm_step": "LBM_STEP",
        "m_voxelize": "VOXELIZE",
        "m_heat": "HEAT",
        "m_particles": "PARTICLES_SIM",
        "m_stream": "STREAM_SIM",
        "m_render": "RENDER",
        "m_blur": "BLUR",
        "m_present": "PRESENT",
        "m_taa": "TAA",
        "m_pdraw": "PARTICLES_DRAW",
        "m_sdraw": "STREAM_DRAW",
        "m_mesh": "MESH_DRAW",
    }
    os.makedirs(OUT, exist_ok=True)
    chunks = [
        "// Generated by oracle/wgsl_translate.py from the reference's shader sources.\n"
        "// Build output only; not part of the repository.\n"
    ]
    for ns, const in mods.items():
        wgsl = resolve(const, table, rig)
        open(os.path.join(OUT, f"{const.lower()}.wgsl"), "w").write(wgsl)
        chunks.append(translate_module(ns, wgsl, report))
    open(os.path.join(OUT, "wgsl_modules.inc"), "w").write("\n".join(chunks))
    with open(os.path.join(OUT, "translate_report.txt"), "w") as f:
        f.write("AbstractFloat literal folds:\n" + "\n".join(report) + "\n")
    print("wrote", os.path.join(OUT, "wgsl_modules.inc"), "folds:", report)


if __name__ == "__main__":
    main()
