"""Mechanical WGSL -> C++ translation of the reference shaders.

TEST INFRASTRUCTURE.  This script reads the reference's own shader sources
(shaders/common.wgsl, film.wgsl, strata.wgsl, km.wgsl, cure.wgsl, shade.wgsl,
deposit.wgsl)
from the reference checkout and rewrites them token by token into C++ that
compiles against wgsl_rt.hpp.  The output goes to oracle/_ref/ (git-ignored):
no reference source is stored in this repository.  The translated shaders,
driven by driver.cpp in the dispatch order of Film::encode_frame, are the
strongest available stand-in for the reference (whose Rust/wgpu host cannot be
built or run here); they pin the hand-written oracle through the fixtures in
tests/golden/.

Only the subset of WGSL that these shaders use is handled: structs, module
constants and bindings, functions, let/var, if/else/for/while, vector and
array constructors, swizzles, pointers to function variables, atomics and
barriers (the driver emulates workgroup phases where a barrier matters).
`switch` becomes an if / else-if chain.  Helpers whose workgroup barriers
sit inside them are left to driver.cpp (DRIVER_PROVIDED).

Usage: python translate.py <reference_root> <out_file> [real]
  real = double (default) or float: the C++ type that WGSL f32 maps to.
"""
import re
import sys

MODULES = ["common.wgsl", "film.wgsl", "strata.wgsl", "km.wgsl", "cure.wgsl", "shade.wgsl", "deposit.wgsl"]


def split_items(src):
    """Split WGSL source into top-level items (text chunks)."""
    items, i, n = [], 0, len(src)
    while i < n:
        while i < n and src[i].isspace():
            i += 1
        if i >= n:
            break
        if src.startswith("//", i):
            j = src.find("\n", i)
            i = n if j < 0 else j + 1
            continue
        start, depth = i, 0
        while i < n:
            ch = src[i]
            if ch == "{":
                depth += 1
            elif ch == "}":
                depth -= 1
                if depth == 0:
                    i += 1
                    break
            elif ch == ";" and depth == 0:
                i += 1
                break
            i += 1
        items.append(src[start:i].strip())
    return items


def item_name(it):
    s = re.sub(r"@\w+(\([^)]*\))?\s*", "", it).strip()
    m = re.match(r"(fn|struct|const|var(?:<[^>]*>)?|override)\s+(\w+)", s)
    return (m.group(1), m.group(2)) if m else (None, None)


def split_top(s, sep=","):
    """Split on `sep` at bracket depth 0 (parens, angle brackets, squares)."""
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch in "(<[":
            depth += 1
        elif ch in ")>]":
            depth -= 1
        if ch == sep and depth == 0:
            out.append(cur)
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur)
    return [x.strip() for x in out]


def conv_type(t):
    t = t.strip()
    m = re.fullmatch(r"ptr<\s*function\s*,\s*(.+)>", t)
    if m:
        return conv_type(m.group(1)) + "*"
    m = re.fullmatch(r"atomic<\s*(\w+)\s*>", t)
    if m:
        return m.group(1)
    m = re.fullmatch(r"array<(.+)>", t)
    if m:
        parts = split_top(m.group(1))
        if len(parts) == 1:
            return "RtBuf<%s>" % conv_type(parts[0])
        return "array<%s, %s>" % (conv_type(parts[0]), parts[1])
    m = re.fullmatch(r"(vec[234])<\s*(\w+)\s*>", t)
    if m:
        return "%s<%s>" % (m.group(1), m.group(2))
    if t.startswith("texture_storage_2d"):
        return "Tex"
    return t


FLOAT_LIT = re.compile(r"(?<![\w.])((?:\d+\.\d*|\.\d+)(?:[eE][+-]?\d+)?|\d+[eE][+-]?\d+)(?![\w.])")


def conv_literals(code):
    def rep(m):
        lit = m.group(1)
        if lit.endswith("."):
            lit += "0"
        return "f32(%sf)" % lit
    return FLOAT_LIT.sub(rep, code)


def conv_array_ctor(code):
    """array<T, N>(a, b) -> make_array<T, N>(a, b)"""
    return re.sub(r"(?<![\w:<])array<([^()]*?)>\(", r"make_array<\1>(", code)


def conv_switch(code):
    """switch e { case a, b: {..} default: {..} } -> an if / else-if chain."""
    while True:
        m = re.search(r"\bswitch\s+(.+?)\s*\{", code)
        if not m:
            return code
        end = match_bracket(code, m.end() - 1)
        inner = code[m.end():end - 1]
        arms, i = [], 0
        while True:
            c = re.compile(r"\s*(case\s+(.+?)|default)\s*:\s*\{", re.S).match(inner, i)
            if not c:
                assert not inner[i:].strip(), inner[i:][:60]
                break
            close = match_bracket(inner, c.end() - 1)
            arms.append((None if c.group(1) == "default" else split_top(c.group(2)), inner[c.end():close - 1]))
            i = close
        parts = []
        for k, (labels, body) in enumerate(arms):
            if labels is None:
                parts.append("{" + body + "}")
            else:
                cond = " || ".join("__sw == (%s)" % lab for lab in labels)
                parts.append("if (%s) {%s}" % (cond, body))
        chain = " else ".join(parts)
        code = code[:m.start()] + "{ const auto __sw = (%s); %s }" % (m.group(1), chain) + code[end:]


def conv_body(body):
    body = conv_switch(body)
    out = []
    for line in body.split("\n"):
        s = line
        s = re.sub(r"\blet\s+(\w+)\s*:\s*([^=;]+?)\s*=", lambda m: "const %s %s =" % (conv_type(m.group(2)), m.group(1)), s)
        s = re.sub(r"\bvar\s+(\w+)\s*:\s*([^=;]+?)\s*=", lambda m: "%s %s =" % (conv_type(m.group(2)), m.group(1)), s)
        s = re.sub(r"\bvar\s+(\w+)\s*:\s*([^=;]+?)\s*;", lambda m: "%s %s{};" % (conv_type(m.group(2)), m.group(1)), s)
        s = re.sub(r"\b(let|var)\s+(\w+)\s*=", r"auto \2 =", s)
        s = re.sub(r"\bif\s+(?!\()(.+?)\s*\{", r"if (\1) {", s)
        s = re.sub(r"\bif\s+(\(.+?)\s*\{", lambda m: "if (%s) {" % m.group(1), s)
        s = re.sub(r"\bwhile\s+(.+?)\s*\{", r"while (\1) {", s)
        s = re.sub(r"\.([xyzw]{2,4})\b", r".\1()", s)
        s = re.sub(r"ptr<\s*function\s*,\s*(\w+)\s*>", r"\1*", s)
        out.append(s)
    code = "\n".join(out)
    code = conv_array_ctor(code)
    code = conv_literals(code)
    return code


def conv_fn(it, name):
    it = re.sub(r"@compute\s*@workgroup_size\([^)]*\)\s*", "", it)
    it = re.sub(r"^\s*@(fragment|vertex)\s*", "", it)  # stage attributes of render entry points
    m = re.match(r"fn\s+(\w+)\s*\((.*?)\)\s*(->\s*(?:@\w+\([^)]*\)\s*)?([^{]+?))?\s*\{", it, re.S)
    assert m, it[:80]
    params = []
    for p in split_top(m.group(2)):
        p = re.sub(r"@\w+\([^)]*\)\s*", "", p).strip()
        pn, pt = p.split(":", 1)
        params.append("%s %s" % (conv_type(pt), pn.strip()))
    ret = conv_type(m.group(4)) if m.group(4) else "void"
    body = it[m.end():]
    proto = "%s %s(%s)" % (ret, name, ", ".join(params))
    return proto, proto + " {" + conv_body(body)


def conv_struct(it, name):
    m = re.match(r"struct\s+\w+\s*\{(.*)\}", it, re.S)
    fields = []
    for f in split_top(m.group(1)):
        if not f:
            continue
        fn_, ft = f.split(":", 1)
        fields.append("    %s %s{};" % (conv_type(ft), fn_.strip()))
    return "struct %s {\n%s\n};" % (name, "\n".join(fields))


def conv_global(it, kind, name):
    s = re.sub(r"@\w+\([^)]*\)\s*", "", it).strip().rstrip(";")
    if kind == "const":
        m = re.match(r"const\s+(\w+)\s*:\s*(.+?)\s*=\s*(.+)$", s, re.S)
        return "constexpr %s %s = %s;" % (conv_type(m.group(2)), m.group(1), conv_literals(m.group(3)))
    m = re.match(r"var(?:<[^>]*>)?\s+(\w+)\s*:\s*(.+)$", s, re.S)
    return "%s %s{};" % (conv_type(m.group(2)), m.group(1))


# Dispatches whose invocations read neighbour values that the same dispatch
# writes.  Their reads are redirected to `<name>__old`, a snapshot the driver
# takes before the dispatch (Jacobi semantics, as in the oracle).
JACOBI = {"nose": ["delta"], "strata_fill": ["strata_h", "strata_pig", "strata_cure"]}

# Entry points whose workgroup barriers matter: emitted as one function per
# barrier-separated phase (`<name>__p0`, `__p1`, ...).
PHASED = ["mark_tiles"]

# Helpers with workgroup barriers inside them: only their prototypes are
# emitted; driver.cpp gives them workgroup-at-a-time definitions (the driver
# runs a workgroup's invocations one after the other, then completes the
# barrier's work: the tile's moved flag, the tree sums of wg_reduce and
# total_parts in the shader's order).
DRIVER_PROVIDED = {"begin_motion", "end_motion", "wg_reduce", "total_parts"}

# Entry points not translated: cg_reduce_mass keeps its barriers inline
# (driver.cpp restates its two tree sums); pool8 and the slump pass are not
# on the path.
DROPPED = {"cg_reduce_mass"}


def match_bracket(s, i):
    """Index just past the bracket group that opens at s[i]."""
    pairs = {"[": "]", "(": ")", "{": "}"}
    close, depth = pairs[s[i]], 0
    for j in range(i, len(s)):
        if s[j] == s[i]:
            depth += 1
        elif s[j] == close:
            depth -= 1
            if depth == 0:
                return j + 1
    raise ValueError("unbalanced")


def alias_reads(body, names):
    out, i = "", 0
    pat = re.compile(r"\b(%s)\[" % "|".join(names))
    while True:
        m = pat.search(body, i)
        if not m:
            return out + body[i:]
        end = match_bracket(body, m.end() - 1)
        rest = body[end:].lstrip()
        is_write = rest.startswith("=") and not rest.startswith("==")
        out += body[i:m.start()] + (m.group(1) if is_write else m.group(1) + "__old")
        i = m.end(1)


def phase_split(proto, body):
    """Split a function body at top-level workgroupBarrier() statements."""
    inner = body[body.index("{") + 1: body.rindex("}")]
    parts, depth, cur, i = [], 0, "", 0
    while i < len(inner):
        if inner.startswith("workgroupBarrier();", i) and depth == 0:
            parts.append(cur)
            cur = ""
            i += len("workgroupBarrier();")
            continue
        ch = inner[i]
        depth += ch == "{"
        depth -= ch == "}"
        cur += ch
        i += 1
    parts.append(cur)
    name = re.match(r"\w+\s+(\w+)\(", proto).group(1)
    texts = []
    for k, p in enumerate(parts):
        texts.append(proto.replace(name + "(", "%s__p%d(" % (name, k), 1) + " {" + p + "}")
    return texts


def translate(ref_root, real="double"):
    src = ""
    for mod in MODULES:
        with open("%s/shaders/%s" % (ref_root, mod)) as f:
            src += "\n" + f.read() + "\n"
    items = split_items(src)
    named = [(it,) + item_name(it) for it in items]
    dropped = set(DROPPED)
    changed = True
    while changed:
        changed = False
        for it, kind, nm in named:
            if nm in dropped or kind is None:
                continue
            body_ids = set(re.findall(r"\b\w+\b", it)) - {nm}
            if body_ids & dropped:
                dropped.add(nm)
                changed = True
    structs, globals_, consts, protos, fns, seen = [], [], [], [], [], set()
    for it, kind, nm in named:
        if kind is None or nm in dropped:
            continue
        if nm in seen:
            raise SystemExit("duplicate top-level name %s" % nm)
        seen.add(nm)
        if kind == "struct":
            structs.append(conv_struct(it, nm))
        elif kind == "const":
            consts.append(conv_global(it, kind, nm))
        elif kind.startswith("var"):
            globals_.append(conv_global(it, kind, nm))
        elif kind == "fn":
            if nm in JACOBI:
                it = alias_reads(it, JACOBI[nm])
            proto, text = conv_fn(it, nm)
            protos.append(proto + ";")
            if nm in DRIVER_PROVIDED:
                continue
            fns.append(text)
            if nm in PHASED:
                fns.extend(phase_split(proto, text))
    hdr = [
        "// GENERATED by oracle/wgsl_ref/translate.py from the reference shaders; do not commit.",
        "// f32 -> %s" % real,
        "namespace wg {",
        "using f32 = %s;" % real,
        "#include \"wgsl_rt_types.inc\"",
    ]
    olds = []
    for nm, bufs in JACOBI.items():
        for b in bufs:
            decl = [g for g in globals_ if re.search(r"\b%s\{\};$" % b, g)][0]
            olds.append(decl.replace(" %s{};" % b, " %s__old{};" % b))
    out = hdr + consts + structs + globals_ + olds + protos + fns + ["}  // namespace wg", ""]
    out.append("// dropped: " + " ".join(sorted(dropped)))
    return "\n".join(out) + "\n"


RGBA = {"r": "x", "g": "y", "b": "z", "a": "w"}


def translate_subset(ref_root, module, roots, stubs, namespace, real="double", members=()):
    """Translate the functions `roots` of one shader module and everything they
    call, into their own namespace; the functions in `stubs` get empty bodies
    (the driver never reaches them).  Colour swizzles (.rgb, .a) map to xyzw,
    except on the variables named in `members`, whose fields are called a, b,
    c (a uniform struct such as resolve.wgsl's Res)."""
    with open("%s/shaders/%s" % (ref_root, module)) as f:
        src = f.read()
    items = split_items(src)
    named = {nm: (it, kind) for it, kind, nm in ((it,) + item_name(it) for it in items) if nm}
    fns = {nm for nm, (it, kind) in named.items() if kind == "fn"}
    need, todo = set(), list(roots)
    while todo:
        nm = todo.pop()
        if nm in need:
            continue
        need.add(nm)
        if nm in stubs:
            continue
        ids = set(re.findall(r"\b\w+\b", named[nm][0])) - {nm}
        todo.extend(sorted(ids & fns))
    consts, structs, globals_, protos, bodies = [], [], [], [], []
    for it, kind, nm in ((it,) + item_name(it) for it in items):
        if kind is None:
            continue
        if kind == "const":
            consts.append(conv_global(it, kind, nm).replace("constexpr ", "const ", 1))
        elif kind == "struct":
            structs.append(conv_struct(re.sub(r"@\w+(\([^)]*\))?\s*", "", it), nm))
        elif kind.startswith("var"):
            g = conv_global(it, kind, nm)
            g = g.replace("texture_2d<f32>", "Tex").replace("sampler ", "Sampler ")
            globals_.append(g)
        elif kind == "fn" and nm in need:
            it2 = re.sub(r"(\b\w+)?\.([rgba]{1,4})\b",
                         lambda m: m.group(0) if m.group(1) in members
                         else (m.group(1) or "") + "." + "".join(RGBA[ch] for ch in m.group(2)), it)
            proto, text = conv_fn(it2, nm)
            protos.append(proto + ";")
            if nm in stubs:
                ret = proto.split(" ", 1)[0]
                bodies.append(proto + " { return %s{}; }" % ret if ret != "void" else proto + " {}")
            else:
                bodies.append(text)
    hdr = ["// GENERATED by oracle/wgsl_ref/translate.py from the reference shaders; do not commit.",
           "namespace %s {" % namespace, "using f32 = %s;" % real, "#include \"wgsl_rt_types.inc\""]
    out = hdr + consts + structs + globals_ + protos + bodies + ["}  // namespace %s" % namespace, ""]
    out.append("// translated: " + " ".join(sorted(need)) + "; stubs: " + " ".join(sorted(set(stubs) & need)))
    return "\n".join(out) + "\n"


if __name__ == "__main__":
    ref, dst = sys.argv[1], sys.argv[2]
    real = sys.argv[3] if len(sys.argv) > 3 else "double"
    with open(dst, "w") as f:
        f.write(translate(ref, real))
