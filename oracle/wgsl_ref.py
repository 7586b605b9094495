"""Mechanical WGSL -> C++ translation of a compute shader, built and run on the CPU.

Test infrastructure only. It turns the reference's own raycast shader
(woxel: src/shaders/raycast.comp.wgsl) into C++ that runs each invocation of the
compute entry point on the host, so the C oracle (woxel_oracle.c, a hand-written
restatement of the same shader) can be checked against the shader source itself:
control flow, constants, index arithmetic and the order of every FP32 operation come
from the shader text, not from a second reading of it. What WGSL leaves to the
implementation (NaN in min/max, normalize, dot order, mix, rgba8unorm rounding,
float-to-int conversion) is pinned in wgsl_rt.h to the oracle's choices.

The translation covers the WGSL subset the shader uses: structs, module constants,
uniform / storage buffers, 3D textures and a write-only storage texture, functions,
let / var / const, if / else, for / while / loop, switch, return / break / continue,
vectors with swizzles, arrays, struct constructors and the built-ins of wgsl_rt.h.
Member access is resolved by name (no type inference): a struct member spelled like
a swizzle (x, rgb, ...) is rejected rather than guessed.

Generated files go to oracle/_ref/ (not part of the repository):
    python oracle/wgsl_ref.py [path/to/raycast.comp.wgsl]
builds oracle/_ref/libraycast_wgsl.so. The shader is looked up in the reference
checkout given by WOXEL_REFERENCE (default /root/reference).
"""
from __future__ import annotations

import ctypes as C
import os
import re
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
SHADER_REL = "src/shaders/raycast.comp.wgsl"


def shader_path() -> Path:
    return Path(os.environ.get("WOXEL_REFERENCE", "/root/reference")) / SHADER_REL


# --------------------------------------------------------------------------- tokens
_TOKEN = re.compile(r"""
    (?P<ws>\s+|//[^\n]*|/\*.*?\*/)
  | (?P<num>0[xX][0-9a-fA-F]+[iu]?
       |(?:[0-9]+\.[0-9]*|\.[0-9]+)(?:[eE][+-]?[0-9]+)?[fh]?
       |[0-9]+[eE][+-]?[0-9]+[fh]?
       |[0-9]+[iuf]?)
  | (?P<id>[A-Za-z_][A-Za-z0-9_]*)
  | (?P<op><<=|>>=|->|<=|>=|==|!=|&&|\|\||<<|>>|\+=|-=|\*=|/=|%=|&=|\|=|\^=|\+\+|--|[{}()\[\]<>;:,.=+\-*/%&|^!~@])
""", re.S | re.X)


def tokenize(src: str) -> list:
    out, pos = [], 0
    while pos < len(src):
        m = _TOKEN.match(src, pos)
        if not m:
            raise SyntaxError(f"wgsl: cannot tokenize at {src[pos:pos + 30]!r}")
        pos = m.end()
        if m.lastgroup != "ws":
            out.append((m.lastgroup, m.group()))
    out.append(("eof", ""))
    return out


# --------------------------------------------------------------------------- parser
TYPE_GENERICS = {"vec2", "vec3", "vec4", "array", "mat2x2", "mat3x3", "mat4x4", "mat4x3", "mat3x4",
                 "texture_3d", "texture_2d", "texture_storage_2d", "texture_storage_3d", "ptr", "atomic"}


class Parser:
    def __init__(self, toks):
        self.t = toks
        self.i = 0

    def peek(self, k=0):
        return self.t[self.i + k]

    def next(self):
        tok = self.t[self.i]
        self.i += 1
        return tok

    def accept(self, val):
        if self.peek()[1] == val:
            self.i += 1
            return True
        return False

    def expect(self, val):
        tok = self.next()
        if tok[1] != val:
            raise SyntaxError(f"wgsl: expected {val!r}, got {tok[1]!r} near token {self.i}")
        return tok

    def ident(self):
        tok = self.next()
        if tok[0] != "id":
            raise SyntaxError(f"wgsl: expected an identifier, got {tok[1]!r}")
        return tok[1]

    # attributes: @name or @name(args)
    def attrs(self):
        out = {}
        while self.accept("@"):
            name = self.ident()
            args = []
            if self.accept("("):
                while not self.accept(")"):
                    args.append(self.expr())
                    self.accept(",")
            out[name] = args
        return out

    def close_angle(self):
        tok = self.peek()
        if tok[1] == ">":
            self.i += 1
        elif tok[1] == ">>":  # split the shift token closing two template lists
            self.t[self.i] = ("op", ">")
        elif tok[1] == ">=":
            self.t[self.i] = ("op", "=")
        else:
            raise SyntaxError(f"wgsl: expected '>' in a template list, got {tok[1]!r}")

    def type_(self):
        name = self.ident()
        params = []
        if name in TYPE_GENERICS and self.peek()[1] == "<":
            self.next()
            while True:
                tok = self.peek()
                if tok[0] == "num":
                    params.append(int(self.next()[1].rstrip("iu"), 0))
                elif tok[0] == "id" and tok[1] in ("read", "write", "read_write", "function", "private",
                                                   "workgroup", "uniform", "storage") or \
                        tok[0] == "id" and re.fullmatch(r"r\w*\d\w*", tok[1]):
                    params.append(self.next()[1])
                else:
                    params.append(self.type_())
                if self.accept(","):
                    if self.peek()[1] in (">", ">>"):
                        break
                    continue
                break
            self.close_angle()
        return ("T", name, params)

    def module(self):
        decls = []
        while self.peek()[0] != "eof":
            at = self.attrs()
            kw = self.peek()[1]
            if kw == "struct":
                self.next()
                name = self.ident()
                self.expect("{")
                members = []
                while not self.accept("}"):
                    mat = self.attrs()
                    mname = self.ident()
                    self.expect(":")
                    members.append((mname, self.type_(), mat))
                    self.accept(",")
                self.accept(";")
                decls.append(("struct", name, members))
            elif kw == "var":
                self.next()
                space = []
                if self.accept("<"):
                    while True:
                        space.append(self.ident())
                        if not self.accept(","):
                            break
                    self.close_angle()
                name = self.ident()
                self.expect(":")
                ty = self.type_()
                init = self.expr() if self.accept("=") else None
                self.expect(";")
                decls.append(("global", name, ty, space, at, init))
            elif kw in ("const", "override", "let"):
                self.next()
                name = self.ident()
                ty = self.type_() if self.accept(":") else None
                self.expect("=")
                e = self.expr()
                self.expect(";")
                decls.append(("gconst", name, ty, e))
            elif kw == "fn":
                self.next()
                name = self.ident()
                self.expect("(")
                params = []
                while not self.accept(")"):
                    pat = self.attrs()
                    pname = self.ident()
                    self.expect(":")
                    params.append((pname, self.type_(), pat))
                    self.accept(",")
                ret = None
                if self.accept("->"):
                    self.attrs()
                    ret = self.type_()
                body = self.block()
                decls.append(("fn", name, params, ret, body, at))
            elif kw == ";":
                self.next()
            else:
                raise SyntaxError(f"wgsl: unexpected {kw!r} at module scope")
        return decls

    def block(self):
        self.expect("{")
        out = []
        while not self.accept("}"):
            out.append(self.stmt())
        return ("block", out)

    def decl_stmt(self):
        kw = self.next()[1]
        if kw == "var" and self.accept("<"):
            while not self.peek()[1] in (">",):
                self.next()
            self.close_angle()
        name = self.ident()
        ty = self.type_() if self.accept(":") else None
        init = self.expr() if self.accept("=") else None
        return (kw, name, ty, init)

    def simple_stmt(self):
        """Assignment, increment, call or declaration (no trailing ';')."""
        kw = self.peek()[1]
        if kw in ("let", "var", "const"):
            return self.decl_stmt()
        if kw == "_" and self.peek(1)[1] == "=":
            self.next()
            self.next()
            return ("expr", self.expr())
        lhs = self.unary()
        op = self.peek()[1]
        if op in ("=", "+=", "-=", "*=", "/=", "%=", "&=", "|=", "^=", "<<=", ">>="):
            self.next()
            return ("assign", op, lhs, self.expr())
        if op in ("++", "--"):
            self.next()
            return ("incdec", op, lhs)
        return ("expr", self.postfix_rest(lhs))

    def stmt(self):
        kw = self.peek()[1]
        if kw == "{":
            return self.block()
        if kw == "if":
            self.next()
            cond = self.expr()
            then = self.block()
            els = None
            if self.accept("else"):
                els = self.stmt() if self.peek()[1] == "if" else self.block()
            return ("if", cond, then, els)
        if kw == "for":
            self.next()
            self.expect("(")
            init = None if self.peek()[1] == ";" else self.simple_stmt()
            self.expect(";")
            cond = None if self.peek()[1] == ";" else self.expr()
            self.expect(";")
            upd = None if self.peek()[1] == ")" else self.simple_stmt()
            self.expect(")")
            return ("for", init, cond, upd, self.block())
        if kw == "while":
            self.next()
            cond = self.expr()
            return ("for", None, cond, None, self.block())
        if kw == "loop":
            self.next()
            self.expect("{")
            body, cont = [], None
            while not self.accept("}"):
                if self.peek()[1] == "continuing":
                    self.next()
                    cont = self.block()
                else:
                    body.append(self.stmt())
            if cont is not None:
                raise SyntaxError("wgsl: 'continuing' blocks are not supported")
            return ("for", None, None, None, ("block", body))
        if kw == "switch":
            self.next()
            sel = self.expr()
            self.expect("{")
            cases = []
            while not self.accept("}"):
                labels = []
                if self.accept("default"):
                    labels.append("default")
                else:
                    self.expect("case")
                    while True:
                        if self.accept("default"):
                            labels.append("default")
                        else:
                            labels.append(self.expr())
                        if not self.accept(","):
                            break
                        if self.peek()[1] in (":", "{"):
                            break
                self.accept(":")
                cases.append((labels, self.block()))
            return ("switch", sel, cases)
        if kw == "return":
            self.next()
            e = None if self.peek()[1] == ";" else self.expr()
            self.expect(";")
            return ("return", e)
        if kw in ("break", "continue", "discard"):
            self.next()
            if kw == "break" and self.peek()[1] == "if":
                raise SyntaxError("wgsl: 'break if' is not supported")
            self.expect(";")
            return (kw,)
        s = self.simple_stmt()
        self.expect(";")
        return s

    # expressions, lowest precedence first
    BIN = [["||"], ["&&"], ["|"], ["^"], ["&"], ["==", "!="], ["<", ">", "<=", ">="], ["<<", ">>"],
           ["+", "-"], ["*", "/", "%"]]

    def expr(self, level=0):
        if level == len(self.BIN):
            return self.unary()
        lhs = self.expr(level + 1)
        while self.peek()[0] == "op" and self.peek()[1] in self.BIN[level]:
            op = self.next()[1]
            lhs = ("bin", op, lhs, self.expr(level + 1))
        return lhs

    def unary(self):
        tok = self.peek()
        if tok[1] in ("-", "!", "~", "&", "*"):
            self.next()
            return ("un", tok[1], self.unary())
        return self.postfix_rest(self.primary())

    def postfix_rest(self, e):
        while True:
            if self.accept("."):
                e = ("member", e, self.ident())
            elif self.accept("["):
                idx = self.expr()
                self.expect("]")
                e = ("index", e, idx)
            else:
                return e

    def primary(self):
        tok = self.peek()
        if tok[0] == "num":
            self.next()
            return ("lit", tok[1])
        if tok[1] == "(":
            self.next()
            e = self.expr()
            self.expect(")")
            return ("paren", e)
        if tok[0] == "id":
            if tok[1] in ("true", "false"):
                self.next()
                return ("bool", tok[1])
            if tok[1] in TYPE_GENERICS and self.peek(1)[1] == "<":
                callee = ("type", self.type_())
            else:
                callee = ("ident", self.next()[1])
            if self.accept("("):
                args = []
                while not self.accept(")"):
                    args.append(self.expr())
                    self.accept(",")
                return ("call", callee, args)
            if callee[0] == "type":
                raise SyntaxError("wgsl: a type used as a value")
            return callee
        raise SyntaxError(f"wgsl: unexpected token {tok[1]!r}")


# --------------------------------------------------------------------------- layout
SCALARS = {"f32": "float", "u32": "uint32_t", "i32": "int32_t", "bool": "bool"}
VEC_N = {"vec2": 2, "vec3": 3, "vec4": 4}


def round_up(a, b):
    return (a + b - 1) // b * b


class Module:
    def __init__(self, decls):
        self.structs = {d[1]: d[2] for d in decls if d[0] == "struct"}
        self.fns = {d[1]: d for d in decls if d[0] == "fn"}
        self.globals = [d for d in decls if d[0] == "global"]
        self.consts = [d for d in decls if d[0] == "gconst"]
        self.member_names = {m[0] for ms in self.structs.values() for m in ms}

    def align_size(self, t, uniform):
        """WGSL AlignOf / SizeOf of a host-shareable type in the uniform or storage space."""
        name, params = t[1], t[2]
        if name in SCALARS:
            return 4, 4
        if name in VEC_N:
            n = VEC_N[name]
            return (8 if n == 2 else 16), 4 * n
        m = re.fullmatch(r"mat(\d)x(\d)", name)
        if m:
            cols, rows = int(m.group(1)), int(m.group(2))
            a = 8 if rows == 2 else 16
            return a, cols * round_up(4 * rows, a)
        if name == "array":
            ea, es = self.align_size(params[0], uniform)
            stride = round_up(es, ea)
            if uniform:
                ea = round_up(ea, 16)
                stride = round_up(stride, 16)
            n = params[1] if len(params) > 1 else 0
            return ea, stride * n
        if name in self.structs:
            off, al = 0, 1
            for _, mt, _ in self.structs[name]:
                a, s = self.align_size(mt, uniform)
                off = round_up(off, a) + s
                al = max(al, a)
            if uniform:
                al = round_up(al, 16)
            return al, round_up(off, al)
        raise TypeError(f"wgsl: no host-shareable layout for {name}")

    def stride(self, t, uniform):
        a, s = self.align_size(t, uniform)
        return round_up(s, a)


# --------------------------------------------------------------------------- emitter
CPP_RESERVED = {"auto", "break", "case", "char", "class", "const", "continue", "default", "delete", "do",
                "double", "else", "enum", "extern", "float", "for", "goto", "if", "int", "long", "new",
                "operator", "private", "public", "register", "return", "short", "signed", "sizeof",
                "static", "struct", "switch", "template", "this", "throw", "try", "typedef", "union",
                "unsigned", "virtual", "void", "volatile", "while", "and", "or", "not", "xor", "bool",
                "true", "false", "namespace", "using", "typename", "friend", "inline", "mutable",
                "explicit", "export", "protected", "catch", "asm", "wgsl", "std", "main"}
BUILTINS = {"min", "max", "floor", "trunc", "abs", "sqrt", "dot", "length", "normalize", "mix", "select",
            "all", "any", "textureLoad", "textureStore", "textureDimensions", "arrayLength"}
SWIZ = {"x": 0, "y": 1, "z": 2, "w": 3, "r": 0, "g": 1, "b": 2, "a": 3}


def cname(n):
    return n + "_" if n in CPP_RESERVED else n


class Emitter:
    def __init__(self, mod: Module):
        self.m = mod
        self.resource_kinds = {}
        for g in mod.globals:
            self.resource_kinds[g[1]] = g

    def ctype(self, t):
        name, params = t[1], t[2]
        if name in SCALARS:
            return SCALARS[name]
        if name in VEC_N:
            return f"wgsl::Vec<{self.ctype(params[0])}, {VEC_N[name]}>"
        m = re.fullmatch(r"mat(\d)x(\d)", name)
        if m:
            return f"std::array<wgsl::Vec<{self.ctype(params[0])}, {m.group(2)}>, {m.group(1)}>"
        if name == "array":
            if len(params) < 2:
                return f"wgsl::Storage<{self.ctype(params[0])}>"
            return f"std::array<{self.ctype(params[0])}, {params[1]}>"
        if name == "texture_3d":
            return f"wgsl::Tex3<{self.ctype(params[0])}>"
        if name == "texture_storage_2d":
            if params[0] != "rgba8unorm":
                raise TypeError(f"wgsl: storage texture format {params[0]} is not supported")
            return "wgsl::TexStore2"
        if name in self.m.structs:
            return "S_" + name
        raise TypeError(f"wgsl: type {name} is not supported")

    # literals: abstract floats become f32, suffix u -> uint32_t, i / none -> int32_t
    def lit(self, s):
        if s.endswith("h"):
            raise TypeError("wgsl: f16 literals are not supported")
        is_float = s.endswith("f") and not s.lower().startswith("0x") or "." in s or \
            (("e" in s or "E" in s) and not s.lower().startswith("0x"))
        if is_float:
            body = s[:-1] if s.endswith("f") else s
            if body.endswith("."):
                body += "0"
            if body.startswith("."):
                body = "0" + body
            return f"{body}f"
        if s.endswith("u"):
            return f"uint32_t({s[:-1]}u)"
        if s.endswith("i"):
            return f"int32_t({s[:-1]})"
        return f"int32_t({s})"

    def expr(self, e):
        k = e[0]
        if k == "lit":
            return self.lit(e[1])
        if k == "bool":
            return e[1]
        if k == "paren":
            return f"({self.expr(e[1])})"
        if k == "ident":
            return cname(e[1])
        if k == "un":
            if e[1] == "&":  # pointers: only as arrayLength(&buffer)
                return self.expr(e[2])
            if e[1] == "*":
                return self.expr(e[2])
            return f"({e[1]}{self.expr(e[2])})"
        if k == "bin":
            op, a, b = e[1], self.expr(e[2]), self.expr(e[3])
            if op == "%":
                return f"wgsl::mod({a}, {b})"
            if op in ("&", "|", "^"):
                return f"wgsl::{ {'&': 'band', '|': 'bor', '^': 'bxor'}[op] }({a}, {b})"
            if op == "<<":
                return f"wgsl::shl({a}, {b})"
            if op == ">>":
                return f"wgsl::shr({a}, {b})"
            return f"({a} {op} {b})"
        if k == "member":
            name = e[2]
            obj = self.expr(e[1])
            if name in self.m.member_names:  # struct member (the shader names none like a swizzle)
                if all(c in "xyzw" for c in name) or all(c in "rgba" for c in name):
                    raise TypeError(f"wgsl: member {name} could also be a swizzle")
                return f"{obj}.{cname(name)}"
            if all(c in "xyzw" for c in name) or all(c in "rgba" for c in name):
                idx = [SWIZ[c] for c in name]
                if len(idx) == 1:
                    return f"{obj}.c[{idx[0]}]"
                return f"wgsl::swz<{', '.join(map(str, idx))}>({obj})"
            raise TypeError(f"wgsl: unknown member {name}")
        if k == "index":
            return f"{self.expr(e[1])}[{self.expr(e[2])}]"
        if k == "call":
            return self.call(e[1], e[2])
        raise TypeError(f"wgsl: expression {k} is not supported")

    def call(self, callee, args):
        a = [self.expr(x) for x in args]
        if callee[0] == "type":
            t = callee[1]
            name, params = t[1], t[2]
            if name in VEC_N:
                return f"wgsl::vec<{self.ctype(params[0])}, {VEC_N[name]}>({', '.join(a)})"
            if name == "array":
                et = self.ctype(params[0])
                return f"{self.ctype(t)}{{{{{', '.join(f'wgsl::cvt<{et}>({x})' for x in a)}}}}}"
            raise TypeError(f"wgsl: constructor of {name} is not supported")
        name = callee[1]
        if name in VEC_N:
            if not a:
                raise TypeError("wgsl: vecN() needs arguments or a component type")
            return f"wgsl::vec_auto<{VEC_N[name]}>({', '.join(a)})"
        if name in SCALARS:
            return f"wgsl::cvt<{SCALARS[name]}>({a[0]})" if a else f"{SCALARS[name]}()"
        if name in self.m.structs:
            return f"make_{name}({', '.join(a)})" if a else f"S_{name}{{}}"
        if name in self.m.fns:
            return f"{cname(name)}({', '.join(a)})"
        if name in BUILTINS:
            return f"wgsl::{name}({', '.join(a)})"
        raise TypeError(f"wgsl: unknown function {name}")

    def stmt(self, s, ind):
        p = "    " * ind
        k = s[0]
        if k == "block":
            inner = "".join(self.stmt(x, ind + 1) for x in s[1])
            return f"{p}{{\n{inner}{p}}}\n"
        if k in ("let", "var", "const"):
            _, name, ty, init = s
            t = self.ctype(ty) if ty is not None else "auto"
            q = "const " if k in ("let", "const") else ""
            if init is None:
                return f"{p}{t} {cname(name)}{{}};\n"
            if ty is not None:
                return f"{p}{q}{t} {cname(name)} = static_cast<{t}>({self.expr(init)});\n"
            return f"{p}{q}auto {cname(name)} = {self.expr(init)};\n"
        if k == "assign":
            _, op, lhs, rhs = s
            l, r = self.expr(lhs), self.expr(rhs)
            if op in ("%=", "&=", "|=", "^=", "<<=", ">>="):
                fn = {"%=": "mod", "&=": "band", "|=": "bor", "^=": "bxor", "<<=": "shl", ">>=": "shr"}[op]
                return f"{p}{l} = wgsl::{fn}({l}, {r});\n"
            return f"{p}{l} {op} {r};\n"
        if k == "incdec":
            return f"{p}{self.expr(s[2])}{s[1]};\n"
        if k == "expr":
            return f"{p}(void)({self.expr(s[1])});\n"
        if k == "return":
            return f"{p}return;\n" if s[1] is None else f"{p}return {self.expr(s[1])};\n"
        if k in ("break", "continue"):
            return f"{p}{k};\n"
        if k == "discard":
            raise TypeError("wgsl: discard in a compute shader")
        if k == "if":
            _, cond, then, els = s
            out = f"{p}if ({self.expr(cond)})\n{self.stmt(then, ind)}"
            if els is not None:
                out += f"{p}else\n{self.stmt(els, ind)}"
            return out
        if k == "for":
            _, init, cond, upd, body = s
            i = self.stmt(init, 0).strip().rstrip(";") if init else ""
            c = self.expr(cond) if cond is not None else ""
            u = self.stmt(upd, 0).strip().rstrip(";") if upd else ""
            if u.startswith("(void)("):
                u = u[len("(void)"):]
            return f"{p}for ({i}; {c}; {u})\n{self.stmt(body, ind)}"
        if k == "switch":
            _, sel, cases = s
            out = f"{p}switch ({self.expr(sel)}) {{\n"
            for labels, body in cases:
                for lab in labels:
                    out += f"{p}default:\n" if lab == "default" else f"{p}case {self.expr(lab)}:\n"
                out += self.stmt(body, ind + 1) + f"{p}    break;\n"
            return out + f"{p}}}\n"
        raise TypeError(f"wgsl: statement {k} is not supported")

    def const_expr(self, e):
        return self.expr(e)

    # struct order: members before the structs that contain them
    def struct_order(self):
        seen, order = set(), []

        def deps(t):
            if t[1] in self.m.structs:
                yield t[1]
            for q in t[2]:
                if isinstance(q, tuple):
                    yield from deps(q)

        def visit(n):
            if n in seen:
                return
            seen.add(n)
            for _, mt, _ in self.m.structs[n]:
                for d in deps(mt):
                    visit(d)
            order.append(n)

        for n in self.m.structs:
            visit(n)
        return order

    def loader(self, t, uniform, off_expr):
        """C++ expression loading a value of type t from `p + off` with the WGSL layout."""
        name, params = t[1], t[2]
        if name in SCALARS:
            if name == "bool":
                return f"(wgsl::load_scalar<uint32_t>(p + {off_expr}) != 0u)"
            return f"wgsl::load_scalar<{SCALARS[name]}>(p + {off_expr})"
        if name in VEC_N:
            et = self.ctype(params[0])
            comps = ", ".join(self.loader(params[0], uniform, f"{off_expr} + {4 * i}") for i in range(VEC_N[name]))
            return f"wgsl::Vec<{et}, {VEC_N[name]}>{{{{{comps}}}}}"
        m = re.fullmatch(r"mat(\d)x(\d)", name)
        if m:
            cols, rows = int(m.group(1)), int(m.group(2))
            a = 8 if rows == 2 else 16
            colt = ("T", f"vec{rows}", params)
            cs = ", ".join(self.loader(colt, uniform, f"{off_expr} + {c * round_up(4 * rows, a)}") for c in range(cols))
            return f"{self.ctype(t)}{{{{{cs}}}}}"
        if name == "array":
            st = self.m.stride(params[0], uniform)
            if uniform:
                st = round_up(st, 16)
            if params[0][1] in ("f32", "u32", "i32") and st == 4:
                return f"wgsl::load_array<{self.ctype(params[0])}, {params[1]}>(p + {off_expr})"
            es = ", ".join(self.loader(params[0], uniform, f"{off_expr} + {i * st}") for i in range(params[1]))
            return f"{self.ctype(t)}{{{{{es}}}}}"
        if name in self.m.structs:
            return f"shader::load_{name}_{'u' if uniform else 's'}(p + {off_expr})"
        raise TypeError(f"wgsl: cannot load {name}")

    def struct_loaders(self, uniform):
        out = []
        for n in self.struct_order():
            try:
                self.m.align_size(("T", n, []), uniform)
            except TypeError:
                continue
            off, parts = 0, []
            for mname, mt, _ in self.m.structs[n]:
                a, s = self.m.align_size(mt, uniform)
                off = round_up(off, a)
                parts.append(f"    r.{cname(mname)} = {self.loader(mt, uniform, str(off))};\n")
                off += s
            sfx = "u" if uniform else "s"
            out.append(f"[[maybe_unused]] static S_{n} load_{n}_{sfx}(const uint8_t *p) {{\n    S_{n} r{{}};\n"
                       + "".join(parts) + "    return r;\n}\n")
        return "".join(out)

    def emit(self, entry: str):
        m = self.m
        o = ["// Generated by oracle/wgsl_ref.py from the reference's compute shader. Do not edit.\n",
             '#include "wgsl_rt.h"\n#include <thread>\n#include <vector>\n\nnamespace shader {\n\n']
        for n in self.struct_order():
            o.append(f"struct S_{n} {{\n")
            for mname, mt, _ in m.structs[n]:
                o.append(f"    {self.ctype(mt)} {cname(mname)}{{}};\n")
            o.append("};\n")
            args = ", ".join(f"{self.ctype(mt)} a{i}" for i, (_, mt, _) in enumerate(m.structs[n]))
            sets = "".join(f" r.{cname(mn)} = a{i};" for i, (mn, _, _) in enumerate(m.structs[n]))
            o.append(f"[[maybe_unused]] static S_{n} make_{n}({args}) {{ S_{n} r;{sets} return r; }}\n\n")
        o.append(self.struct_loaders(True))
        o.append(self.struct_loaders(False))
        # resources
        for g in m.globals:
            _, name, ty, space, at, init = g
            o.append(f"static {self.ctype(ty)} {cname(name)}{{}};\n")
        for c in m.consts:
            _, name, ty, e = c
            t = self.ctype(ty) if ty is not None else "auto"
            if ty is not None:
                o.append(f"static const {t} {cname(name)} = static_cast<{t}>({self.const_expr(e)});\n")
            else:
                o.append(f"static const auto {cname(name)} = {self.const_expr(e)};\n")
        o.append("\n")
        # forward declarations, then bodies
        sigs = {}
        for name, f in m.fns.items():
            _, _, params, ret, body, at = f
            rt = self.ctype(ret) if ret is not None else "void"
            ps = ", ".join(f"{self.ctype(pt)} {cname(pn)}" for pn, pt, _ in params)
            sigs[name] = f"static {rt} {cname(name)}({ps})"
            o.append(sigs[name] + ";\n")
        o.append("\n")
        for name, f in m.fns.items():
            o.append(sigs[name] + "\n" + self.stmt(f[4], 0) + "\n")
        o.append("}  // namespace shader\n\n")
        o.append(self.abi(entry))
        return "".join(o)

    def abi(self, entry):
        """extern "C" binding and dispatch functions."""
        m = self.m
        f = m.fns[entry]
        wg = [int(x[1].rstrip("iu"), 0) for x in f[5].get("workgroup_size", [])]
        wg = (wg + [1, 1, 1])[:3]
        gid = [pn for pn, pt, pat in f[2] if pat.get("builtin") and pat["builtin"][0] == ("ident", "global_invocation_id")]
        if len(gid) != len(f[2]) or len(gid) != 1:
            raise TypeError("wgsl: the entry point must take global_invocation_id only")
        cases = []
        for g in m.globals:
            _, name, ty, space, at, init = g
            grp = int(at["group"][0][1].rstrip("iu"))
            bnd = int(at["binding"][0][1].rstrip("iu"))
            key = grp * 1000 + bnd
            cn = f"shader::{cname(name)}"
            tn = ty[1]
            if space and space[0] == "uniform":
                body = f"{cn} = shader::load_{tn}_u(static_cast<const uint8_t *>(ptr)); return 0;"
            elif space and space[0] == "storage":
                if tn != "array" or len(ty[2]) != 1:
                    raise TypeError("wgsl: storage buffers other than runtime-sized arrays are not supported")
                et = ty[2][0]
                st = m.stride(et, False)
                ld = f"[](const uint8_t *p) {{ return {self.loader(et, False, '0')}; }}"
                body = (f"{cn}.base = static_cast<const uint8_t *>(ptr); {cn}.stride = {st}; "
                        f"{cn}.count = (uint32_t)(bytes / {st}); {cn}.load = {ld}; return 0;")
            elif tn == "texture_3d":
                body = (f"{cn}.data = static_cast<const {self.ctype(ty[2][0])} *>(ptr); {cn}.w = d0; {cn}.h = d1; "
                        f"{cn}.d = d2; return 0;")
            elif tn == "texture_storage_2d":
                body = f"{cn}.data = static_cast<uint8_t *>(const_cast<void *>(ptr)); {cn}.w = d0; {cn}.h = d1; return 0;"
            else:
                raise TypeError(f"wgsl: resource {name} of type {tn} is not supported")
            cases.append(f"        case {key}: {{ {body} }}\n")
        return (
            'extern "C" int wref_bind(uint32_t group, uint32_t binding, const void *ptr, uint64_t bytes,\n'
            "                         uint32_t d0, uint32_t d1, uint32_t d2) {\n"
            "    (void)bytes; (void)d0; (void)d1; (void)d2;\n"
            "    switch (group * 1000 + binding) {\n" + "".join(cases) +
            "        default: return -1;\n    }\n}\n\n"
            f"// Runs {entry} for every invocation of an nx x ny x nz grid of workgroups of\n"
            f"// {wg[0]}x{wg[1]}x{wg[2]}, rows of workgroups spread over nthreads host threads.\n"
            'extern "C" int wref_dispatch(uint32_t nx, uint32_t ny, uint32_t nz, int nthreads) {\n'
            f"    const uint32_t WX = {wg[0]}, WY = {wg[1]}, WZ = {wg[2]};\n"
            "    auto run = [&](int t, int nt) {\n"
            "        for (uint32_t gz = 0; gz < nz; gz++)\n"
            "            for (uint32_t gy = (uint32_t)t; gy < ny; gy += (uint32_t)nt)\n"
            "                for (uint32_t gx = 0; gx < nx; gx++)\n"
            "                    for (uint32_t lz = 0; lz < WZ; lz++)\n"
            "                        for (uint32_t ly = 0; ly < WY; ly++)\n"
            "                            for (uint32_t lx = 0; lx < WX; lx++)\n"
            f"                                shader::{cname(entry)}(wgsl::Vec<uint32_t, 3>{{{{gx * WX + lx, gy * WY + ly, gz * WZ + lz}}}});\n"
            "    };\n"
            "    if (nthreads < 1) nthreads = 1;\n"
            "    std::vector<std::thread> th;\n"
            "    for (int t = 1; t < nthreads; t++) th.emplace_back(run, t, nthreads);\n"
            "    run(0, nthreads);\n"
            "    for (auto &x : th) x.join();\n"
            "    return 0;\n}\n\n"
            f'extern "C" void wref_workgroup_size(uint32_t *out) {{ out[0] = {wg[0]}; out[1] = {wg[1]}; out[2] = {wg[2]}; }}\n'
            f'extern "C" const char *wref_bindings(void) {{ return "{self.binding_table()}"; }}\n'
        )

    def binding_table(self):
        """name:group:binding:kind;... of the shader's resources."""
        rows = []
        for g in self.m.globals:
            _, name, ty, space, at, init = g
            kind = space[0] if space else ty[1]
            rows.append(f"{name}:{int(at['group'][0][1].rstrip('iu'))}:{int(at['binding'][0][1].rstrip('iu'))}:{kind}")
        return ";".join(rows)


def translate(src: str, entry: str = "cp_main") -> tuple:
    """(C++ source, resource table {name: (group, binding, kind)}) of a WGSL compute shader."""
    mod = Module(Parser(tokenize(src)).module())
    em = Emitter(mod)
    table = {}
    for g in mod.globals:
        _, name, ty, space, at, init = g
        kind = space[0] if space else ty[1]
        table[name] = (int(at["group"][0][1].rstrip("iu")), int(at["binding"][0][1].rstrip("iu")), kind)
    return em.emit(entry), table


def build(src_path: Path | None = None, out_dir: Path = OUT) -> Path:
    """Translate the shader and compile it into out_dir/libraycast_wgsl.so."""
    src_path = Path(src_path) if src_path else shader_path()
    cpp, _ = translate(src_path.read_text())
    out_dir.mkdir(parents=True, exist_ok=True)
    cpp_file = out_dir / "raycast_wgsl.cpp"
    so = out_dir / "libraycast_wgsl.so"
    if not cpp_file.exists() or cpp_file.read_text() != cpp or not so.exists():
        cpp_file.write_text(cpp)
        cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++20", "-fPIC", "-shared", "-pthread",
               "-ffp-contract=off", "-fno-fast-math", "-fno-strict-aliasing", "-fwrapv",
               "-I", str(HERE), "-o", str(so), str(cpp_file)]
        subprocess.run(cmd, check=True)
    return so


class Shader:
    """The translated raycast shader: bind a flattened grid and a uniform, dispatch, read RGBA8."""

    def __init__(self, so: Path | None = None):
        self.so = Path(so) if so else OUT / "libraycast_wgsl.so"
        self.lib = C.CDLL(str(self.so))
        self.lib.wref_bind.argtypes = [C.c_uint32, C.c_uint32, C.c_void_p, C.c_uint64, C.c_uint32, C.c_uint32,
                                       C.c_uint32]
        self.lib.wref_dispatch.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32, C.c_int]
        wg = (C.c_uint32 * 3)()
        self.lib.wref_workgroup_size(wg)
        self.wg = tuple(wg)
        self.lib.wref_bindings.restype = C.c_char_p
        self.table = {}
        for row in self.lib.wref_bindings().decode().split(";"):
            name, g, b, kind = row.split(":")
            self.table[name] = (int(g), int(b), kind)

    def render(self, view: dict, state: bytes, width: int, height: int, nthreads: int = 8):
        """RGBA8 (height, width, 4) of the dispatch wgpu issues for a width x height frame
        (width // 8 x height // 4 workgroups of 8x4); pixels outside stay 0."""
        import numpy as np

        keep = []

        def bind(name, arr, d=(0, 0, 0)):
            g, b, _ = self.table[name]
            a = np.ascontiguousarray(arr)
            keep.append(a)
            rc = self.lib.wref_bind(g, b, a.ctypes.data, a.nbytes, *d)
            if rc != 0:
                raise RuntimeError(f"wref_bind({name}) failed")

        st = np.frombuffer(bytes(state), np.uint8)
        assert st.size == 256
        bind("s", st)
        out = np.zeros((height, width, 4), np.uint8)
        bind("texture", out, (width, height, 1))
        for name, i in (("node5s", 0), ("node4s", 1), ("node3s", 2)):
            bind(name, np.asarray(view["atlas"][i], np.uint32), tuple(int(x) for x in view["dims"][i]))
        for name in ("kids5", "vals5", "kids4", "vals4", "vals3"):
            bind(name, np.asarray(view[name], np.uint32))
        bind("origins", np.asarray(view["origins"], np.int32).reshape(-1, 4))
        self.lib.wref_dispatch(width // self.wg[0], height // self.wg[1], 1, nthreads)
        return out


if __name__ == "__main__":
    p = build(Path(sys.argv[1]) if len(sys.argv) > 1 else None)
    print(p)
