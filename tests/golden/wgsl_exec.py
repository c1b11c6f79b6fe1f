"""Executes the reference's own WGSL on the CPU, to make golden vectors (TEST INFRASTRUCTURE).

ShaderIntel's MPM kernels exist only as WGSL inside JavaScript template strings
(src/physics/mpm.js, src/shaders/linalg.js) and run only in a browser's WebGPU. This module reads
those files, extracts the kernel sources and the modules they import, substitutes the template
values (tile capacity, particles per thread, the portable no-subgroup path, grid DIMS), parses the
WGSL subset they use and runs it:
  - every f32 operation rounds to f32 on its own (numpy float32 scalars and vectors, no FMA);
  - i32 / u32 wrap; integer division truncates; abstract literals take their concrete type where
    WGSL concretises them;
  - a workgroup runs its invocations in index order, switching at each workgroupBarrier, so
    atomics (and the block sort's atomic ranks) resolve in invocation order;
  - builtins WGSL leaves open use one fixed form: mat*vec = (c0*v.x + c1*v.y) + c2*v.z,
    dot = (a.x*b.x + a.y*b.y) + a.z*b.z, length = sqrt(dot), normalize = v / length,
    determinant = first-column cofactor expansion, inverseSqrt = 1/sqrt, max/min ignore NaN;
    log / exp are numpy's f32 functions.
Only tests/golden/gen_golden.py uses it, in a container that has the reference checkout.
"""
import math
import re
import types
import warnings

import numpy as np

warnings.filterwarnings("ignore", category=RuntimeWarning)
f32, i32, u32 = np.float32, np.int32, np.uint32

# ============================================================================ JS template extraction


def template_after(src, start):
    """Returns (body, end) of the JavaScript template literal whose opening backtick is at src[start]."""
    assert src[start] == "`"
    out, k = [], start + 1
    while True:
        c = src[k]
        if c == "\\":
            out.append(src[k:k + 2]); k += 2; continue
        if c == "`":
            return "".join(out), k + 1
        if c == "$" and src[k + 1] == "{":
            depth, j = 1, k + 2
            while depth:
                if src[j] == "`":
                    _, j = template_after(src, j); continue
                if src[j] in "'\"":                      # a quoted JS string: braces inside do not count
                    j = src.index(src[j], j + 1) + 1; continue
                if src[j] == "{":
                    depth += 1
                elif src[j] == "}":
                    depth -= 1
                j += 1
            out.append(src[k:j]); k = j; continue
        out.append(c); k += 1


def field_template(src, anchor, field):
    """The template literal that follows `field:` (and an optional wgsl comment) after `anchor`."""
    a = src.index(anchor)
    m = re.compile(field + r":\s*(/\*\s*wgsl\s*\*/\s*)?([`'])").search(src, a)
    if m.group(2) == "'":                       # a plain single-quoted string
        end = src.index("'", m.end())
        return src[m.end():end]
    return template_after(src, m.end() - 1)[0]


def substitute(tpl, values):
    """Replaces each ${expr} by values[expr] (a string) — the template values of one kernel."""
    out, k = [], 0
    while True:
        j = tpl.find("${", k)
        if j < 0:
            out.append(tpl[k:]); return "".join(out)
        out.append(tpl[k:j])
        depth, e = 1, j + 2
        while depth:
            if tpl[e] == "`":
                _, e = template_after(tpl, e); continue
            if tpl[e] in "'\"":
                e = tpl.index(tpl[e], e + 1) + 1; continue
            depth += {"{": 1, "}": -1}.get(tpl[e], 0)
            e += 1
        expr = tpl[j + 2:e - 1].strip()
        if expr not in values:
            raise KeyError("no value for template expression: " + expr)
        out.append(values[expr])
        k = e


# ============================================================================ runtime values

class Vec:
    __slots__ = ("a",)
    __array_ufunc__ = None          # numpy scalars defer to Vec's reflected operators

    def __init__(self, a):
        self.a = a

    def copy(self):
        return Vec(self.a.copy())

    def __len__(self):
        return len(self.a)

    def _b(self, o):
        return o.a if isinstance(o, Vec) else o

    def __add__(self, o): return Vec(self.a + self._b(o))
    def __radd__(self, o): return Vec(self._b(o) + self.a)
    def __sub__(self, o): return Vec(self.a - self._b(o))
    def __rsub__(self, o): return Vec(self._b(o) - self.a)

    def __mul__(self, o):
        if isinstance(o, Mat):
            raise TypeError("vec * mat not used")
        return Vec(self.a * self._b(o))

    def __rmul__(self, o): return Vec(self._b(o) * self.a)
    def __truediv__(self, o): return Vec(wdiv(self.a, self._b(o)))
    def __rtruediv__(self, o): return Vec(wdiv(self._b(o), self.a))
    def __neg__(self): return Vec(-self.a)
    def __eq__(self, o): return Vec(self.a == self._b(o))
    def __ne__(self, o): return Vec(self.a != self._b(o))
    __hash__ = None
    def __lt__(self, o): return Vec(self.a < self._b(o))
    def __le__(self, o): return Vec(self.a <= self._b(o))
    def __gt__(self, o): return Vec(self.a > self._b(o))
    def __ge__(self, o): return Vec(self.a >= self._b(o))
    def __and__(self, o): return Vec(self.a & self._b(o))
    def __or__(self, o): return Vec(self.a | self._b(o))
    def __lshift__(self, o): return Vec(self.a << self._b(o))
    def __rshift__(self, o): return Vec(self.a >> self._b(o))

    def __getitem__(self, k):
        return self.a[int(k)]

    def __setitem__(self, k, v):
        self.a[int(k)] = v

    def __getattr__(self, name):
        if not name or any(c not in "xyzwrgba" for c in name):
            raise AttributeError(name)
        idx = ["xyzw".index(c) if c in "xyzw" else "rgba".index(c) for c in name]
        if len(idx) == 1:
            return self.a[idx[0]]
        return Vec(self.a[idx].copy())

    def __setattr__(self, name, v):
        if name == "a":
            object.__setattr__(self, name, v)
            return
        idx = ["xyzw".index(c) for c in name]
        if len(idx) == 1:
            self.a[idx[0]] = v
        else:
            self.a[idx] = v.a if isinstance(v, Vec) else v


class Mat:
    """3x3 f32, column-major: m[col][row]."""
    __slots__ = ("c",)
    __array_ufunc__ = None

    def __init__(self, c):
        self.c = c   # (3, 3) float32, c[col, row]

    def copy(self):
        return Mat(self.c.copy())

    def __getitem__(self, k):
        return Vec(self.c[int(k)])      # a view: m[col][row] = v writes through

    def __setitem__(self, k, v):
        self.c[int(k)] = v.a

    def __add__(self, o): return Mat(self.c + o.c)
    def __sub__(self, o): return Mat(self.c - o.c)
    def __neg__(self): return Mat(-self.c)

    def __mul__(self, o):
        if isinstance(o, Mat):
            return Mat(np.stack([matvec(self, Vec(o.c[j])).a for j in range(3)]))
        if isinstance(o, Vec):
            return matvec(self, o)
        return Mat(self.c * o)

    def __rmul__(self, o):
        return Mat(o * self.c)


def matvec(m, v):
    c, x = m.c, v.a
    return Vec(np.array([(c[0, r] * x[0] + c[1, r] * x[1]) + c[2, r] * x[2] for r in range(3)], f32))


def wdiv(a, b):
    """WGSL `/`: float division, or integer division truncating toward zero."""
    if isinstance(a, Vec) or isinstance(b, Vec):
        return Vec(wdiv(a.a if isinstance(a, Vec) else a, b.a if isinstance(b, Vec) else b))
    if isinstance(a, (np.floating, float)) or isinstance(b, (np.floating, float)) or \
            (isinstance(a, np.ndarray) and a.dtype.kind == "f") or (isinstance(b, np.ndarray) and b.dtype.kind == "f"):
        return a / b
    if isinstance(a, int) and isinstance(b, int):
        q = abs(a) // abs(b)
        return q if (a >= 0) == (b >= 0) else -q
    if (isinstance(a, np.ndarray) and a.dtype.kind == "u") or isinstance(a, np.unsignedinteger):
        return a // b
    return (np.trunc(np.asarray(a, np.float64) / np.asarray(b, np.float64))).astype(np.asarray(a).dtype) \
        if isinstance(a, np.ndarray) else type(a)(int(np.trunc(float(a) / float(b))))


def wmod(a, b):
    if isinstance(a, Vec):
        return Vec(wmod(a.a, b.a if isinstance(b, Vec) else b))
    if (isinstance(a, np.ndarray) and a.dtype.kind == "u") or isinstance(a, np.unsignedinteger):
        return a % b
    return a - wdiv(a, b) * b


def cp(v):
    if isinstance(v, (Vec, Mat)):
        return v.copy()
    if isinstance(v, list):
        return [cp(x) for x in v]
    if isinstance(v, types.SimpleNamespace):
        return types.SimpleNamespace(**{k: cp(x) for k, x in vars(v).items()})
    return v


def concrete(v):
    """WGSL concretisation of an abstract literal bound by let/var."""
    if isinstance(v, bool):
        return v
    if isinstance(v, int):
        return i32(v)
    if isinstance(v, float):
        return f32(v)
    return cp(v)


# ---------------------------------------------------------------------------- buffers

class Buffer:
    """A storage buffer: numpy array (N, width) of f32/i32/u32 elements, or struct rows."""

    def __init__(self, arr, kind, width=1, struct=None, struct_types=None):
        self.arr, self.kind, self.width, self.struct = arr, kind, width, struct
        self.struct_types = struct_types or {}

    def __getitem__(self, idx):
        idx = int(idx)
        if self.struct:
            row = self.arr[idx]
            return types.SimpleNamespace(**{n: Vec(row[4 * k:4 * k + 4].copy().view(
                {"u32": u32, "i32": i32}.get(self.struct_types.get(n), row.dtype))) for k, n in enumerate(self.struct)})
        if self.width == 1:
            return self.arr[idx]
        return Vec(self.arr[idx].copy())

    def __setitem__(self, idx, v):
        idx = int(idx)
        if self.struct:
            for k, n in enumerate(self.struct):
                self.arr[idx, 4 * k:4 * k + 4] = getattr(v, n).a.view(self.arr.dtype)
        elif self.width == 1:
            self.arr[idx] = v
        else:
            self.arr[idx] = v.a.view(self.arr.dtype) if v.a.dtype != self.arr.dtype else v.a


# ============================================================================ WGSL parser

TOKEN = re.compile(r"""
    (?P<ws>\s+|//[^\n]*|/\*.*?\*/)
  | (?P<num>0[xX][0-9a-fA-F]+[iu]?|(?:\d+\.\d*|\.\d+|\d+)(?:[eE][+-]?\d+)?[fiuh]?)
  | (?P<id>[A-Za-z_][A-Za-z0-9_]*)
  | (?P<op>->|\+\+|--|\+=|-=|\*=|/=|%=|&=|\|=|\^=|<<=|>>=|<<|>>|<=|>=|==|!=|&&|\|\||[-+*/%<>=!&|^~.,;:(){}\[\]@])
""", re.S | re.X)
TEMPLATED = {"array", "bitcast", "vec2", "vec3", "vec4", "mat3x3", "ptr", "atomic"}


def tokenize(s):
    out, k = [], 0
    while k < len(s):
        m = TOKEN.match(s, k)
        if not m:
            raise SyntaxError("bad WGSL near: " + s[k:k + 40])
        k = m.end()
        if m.lastgroup != "ws":
            out.append((m.lastgroup, m.group()))
    out.append(("eof", ""))
    return out


BIN = {"||": 1, "&&": 2, "|": 3, "^": 4, "&": 5, "==": 6, "!=": 6, "<": 7, ">": 7, "<=": 7, ">=": 7,
       "<<": 8, ">>": 8, "+": 9, "-": 9, "*": 10, "/": 10, "%": 10}


class Parser:
    def __init__(self, src):
        self.t = tokenize(src)
        self.k = 0

    def peek(self, d=0):
        return self.t[self.k + d][1]

    def next(self):
        tok = self.t[self.k]
        self.k += 1
        return tok[1]

    def eat(self, s):
        if self.peek() != s:
            raise SyntaxError(f"expected {s!r}, got {self.peek()!r} at token {self.k}: "
                              + " ".join(x[1] for x in self.t[max(0, self.k - 8):self.k + 8]))
        return self.next()

    def type_(self):
        name = self.next()
        if self.peek() == "<":
            self.next()
            args = []
            while self.peek() != ">":
                args.append(self.type_() if not self.t[self.k][0] == "num" else self.next())
                if self.peek() == ",":
                    self.next()
            self.next()
            return (name, args)
        return (name, [])

    # ---------------------------------------------------------------- top level
    def module(self):
        items = []
        while self.peek() != "":
            p = self.peek()
            if p == "struct":
                self.next(); name = self.next(); self.eat("{")
                fields = []
                while self.peek() != "}":
                    f = self.next(); self.eat(":"); self.type_()
                    fields.append(f)
                    if self.peek() == ",":
                        self.next()
                self.eat("}")
                if self.peek() == ";":
                    self.next()
                items.append(("struct", name, fields))
            elif p == "fn":
                self.next(); name = self.next(); self.eat("(")
                params = []
                while self.peek() != ")":
                    pn = self.next(); self.eat(":"); pt = self.type_()
                    params.append((pn, pt))
                    if self.peek() == ",":
                        self.next()
                self.eat(")")
                rt = None
                if self.peek() == "->":
                    self.next(); rt = self.type_()
                items.append(("fn", name, params, rt, self.block()))
            elif p in ("const", "var", "let"):
                items.append(self.decl())
                self.eat(";")
            elif p == "@":
                while self.peek() == "@":
                    self.next(); self.next()
                    if self.peek() == "(":
                        depth = 0
                        while True:
                            c = self.next(); depth += {"(": 1, ")": -1}.get(c, 0)
                            if depth == 0:
                                break
            else:
                raise SyntaxError("unexpected top-level token " + p)
        return items

    def decl(self):
        kw = self.next()
        space = None
        if kw == "var" and self.peek() == "<":
            self.next(); space = self.next(); self.eat(">")
        name = self.next()
        ty = None
        if self.peek() == ":":
            self.next(); ty = self.type_()
        init = None
        if self.peek() == "=":
            self.next(); init = self.expr()
        return ("decl", kw, space, name, ty, init)

    # ---------------------------------------------------------------- statements
    def block(self):
        self.eat("{")
        out = []
        while self.peek() != "}":
            out.append(self.stmt())
        self.eat("}")
        return out

    def simple(self):
        """A simple statement (no trailing semicolon): decl, assignment, ++/--, or call."""
        if self.peek() in ("let", "var", "const"):
            return self.decl()
        lhs = self.expr()
        op = self.peek()
        if op in ("=", "+=", "-=", "*=", "/=", "%=", "&=", "|=", "^=", "<<=", ">>="):
            self.next()
            return ("assign", op, lhs, self.expr())
        if op in ("++", "--"):
            self.next()
            return ("assign", "+=" if op == "++" else "-=", lhs, ("lit", 1))
        return ("expr", lhs)

    def stmt(self):
        p = self.peek()
        if p == "{":
            return ("block", self.block())
        if p == "if":
            self.next(); self.eat("("); c = self.expr(); self.eat(")")
            body = self.block()
            els = None
            if self.peek() == "else":
                self.next()
                els = [self.stmt()] if self.peek() == "if" else self.block()
            return ("if", c, body, els)
        if p == "for":
            self.next(); self.eat("(")
            init = self.simple() if self.peek() != ";" else None
            self.eat(";")
            cond = self.expr() if self.peek() != ";" else None
            self.eat(";")
            upd = self.simple() if self.peek() != ")" else None
            self.eat(")")
            return ("for", init, cond, upd, self.block())
        if p == "return":
            self.next()
            v = None if self.peek() == ";" else self.expr()
            self.eat(";")
            return ("return", v)
        s = self.simple()
        self.eat(";")
        return s

    # ---------------------------------------------------------------- expressions
    def expr(self, prec=0):
        lhs = self.unary()
        while True:
            op = self.peek()
            p = BIN.get(op)
            if p is None or p <= prec:
                return lhs
            self.next()
            lhs = ("bin", op, lhs, self.expr(p))

    def unary(self):
        p = self.peek()
        if p in ("-", "!", "&", "*", "~"):
            self.next()
            return ("un", p, self.unary())
        return self.postfix(self.primary())

    def primary(self):
        kind, tok = self.t[self.k]
        if kind == "num":
            self.next()
            return ("num", tok)
        if tok == "(":
            self.next(); e = self.expr(); self.eat(")")
            return e
        if kind == "id":
            self.next()
            if tok in ("true", "false"):
                return ("lit", tok == "true")
            targs = None
            if self.peek() == "<" and (tok in TEMPLATED):
                self.next()
                targs = []
                while self.peek() != ">":
                    targs.append(self.type_() if self.t[self.k][0] == "id" else ("num", self.next()))
                    if self.peek() == ",":
                        self.next()
                self.next()
            if self.peek() == "(":
                self.next()
                args = []
                while self.peek() != ")":
                    args.append(self.expr())
                    if self.peek() == ",":
                        self.next()
                self.eat(")")
                return ("call", tok, targs, args)
            return ("name", tok)
        raise SyntaxError("unexpected token " + tok)

    def postfix(self, e):
        while True:
            if self.peek() == ".":
                self.next(); e = ("member", e, self.next())
            elif self.peek() == "[":
                self.next(); i = self.expr(); self.eat("]"); e = ("index", e, i)
            else:
                return e


# ============================================================================ code generation

def num_value(tok):
    t = tok.lower()
    if t.startswith("0x"):
        v = int(t.rstrip("iu"), 16)
        return repr(u32(v)) if t.endswith("u") else (repr(i32(v)) if t.endswith("i") else str(v))
    if t.endswith("u"):
        return f"u32({int(t[:-1])})"
    if t.endswith("i"):
        return f"i32({int(t[:-1])})"
    if t.endswith("f"):
        return f"f32({float(t[:-1])!r})"
    if "." in t or "e" in t:
        return repr(float(t))
    return str(int(t))


class Gen:
    def __init__(self, structs):
        self.structs = structs
        self.lines = []
        self.boxed = set()     # locals whose address is taken (&x): held in a 1-element list

    def emit(self, s, ind):
        self.lines.append("    " * ind + s)

    def e(self, x):
        k = x[0]
        if k == "num":
            return num_value(x[1])
        if k == "lit":
            return repr(x[1])
        if k == "name":
            return f"{x[1]}[0]" if x[1] in self.boxed else x[1]
        if k == "member":
            return f"{self.e(x[1])}.{x[2]}"
        if k == "index":
            return f"{self.e(x[1])}[{self.e(x[2])}]"
        if k == "un":
            op, a = x[1], x[2]
            if op == "-":
                return f"(-{self.e(a)})"
            if op == "!":
                return f"(not {self.e(a)})"
            if op == "~":
                return f"(~{self.e(a)})"
            if op == "*":   # deref of a pointer parameter (a boxed cell)
                return f"{self.e(a)}[0]"
            if op == "&":
                if a[0] == "name":
                    return a[1]            # the cell itself
                raise NotImplementedError("address of " + str(a))
        if k == "bin":
            op, a, b = x[1], self.e(x[2]), self.e(x[3])
            if op == "/":
                return f"wdiv({a}, {b})"
            if op == "%":
                return f"wmod({a}, {b})"
            if op == "&&":
                return f"({a} and {b})"
            if op == "||":
                return f"({a} or {b})"
            return f"({a} {op} {b})"
        if k == "call":
            return self.call(x)
        raise NotImplementedError(str(x))

    def ref(self, x):
        """&buf[idx] -> (buffer expr, index expr) for atomics."""
        assert x[0] == "un" and x[1] == "&", x
        t = x[2]
        if t[0] == "index":
            return self.e(t[1]), self.e(t[2])
        if t[0] == "name":
            return t[1], "None"
        raise NotImplementedError(str(t))

    def call(self, x):
        _, name, targs, args = x
        if name.startswith("atomic"):
            buf, idx = self.ref(args[0])
            rest = ", ".join(self.e(a) for a in args[1:])
            return f"{name}({buf}, {idx}{', ' + rest if rest else ''})"
        if name == "workgroupUniformLoad":
            return f"cp({self.ref(args[0])[0]})"
        if name == "bitcast":
            return f"bitcast({targs[0][0]!r}, {self.e(args[0])})"
        if name == "array":
            return "[" + ", ".join(f"cp({self.e(a)})" for a in args) + "]"
        if name in self.structs:
            fields = self.structs[name]
            return "types.SimpleNamespace(" + ", ".join(f"{f}=cp({self.e(a)})" for f, a in zip(fields, args)) + ")"
        a = ", ".join(self.e(y) for y in args)
        return f"{name}({a})"

    def stmts(self, body, ind):
        if not body:
            self.emit("pass", ind)
        for s in body:
            self.stmt(s, ind)

    def stmt(self, s, ind):
        k = s[0]
        if k == "decl":
            _, kw, space, name, ty, init = s
            if init is not None and init[0] == "call" and init[1] == "workgroupUniformLoad":
                self.emit("yield", ind)   # a workgroup barrier, then the uniform load
            v = self.e(init) if init is not None else f"zero({ty!r})"
            v = f"concrete({v})"
            self.emit(f"{name} = [{v}]" if name in self.boxed else f"{name} = {v}", ind)
        elif k == "assign":
            _, op, lhs, rhs = s
            tgt = self.e(lhs)
            r = self.e(rhs)
            if op == "=":
                self.emit(f"{tgt} = cp({r})", ind)
            else:
                o = op[:-1]
                val = f"wdiv({tgt}, {r})" if o == "/" else (f"wmod({tgt}, {r})" if o == "%" else f"({tgt} {o} {r})")
                self.emit(f"{tgt} = {val}", ind)
        elif k == "expr":
            if s[1][0] == "call" and s[1][1] == "workgroupBarrier":
                self.emit("yield", ind)
            else:
                self.emit(self.e(s[1]), ind)
        elif k == "block":
            self.stmts(s[1], ind)
        elif k == "if":
            self.emit(f"if {self.e(s[1])}:", ind)
            self.stmts(s[2], ind + 1)
            if s[3] is not None:
                self.emit("else:", ind)
                self.stmts(s[3], ind + 1)
        elif k == "for":
            _, init, cond, upd, body = s
            if init:
                self.stmt(init, ind)
            self.emit(f"while {self.e(cond) if cond else 'True'}:", ind)
            self.stmts(body, ind + 1)
            if upd:
                self.stmt(upd, ind + 1)
        elif k == "return":
            self.emit("return" if s[1] is None else f"return {self.e(s[1])}", ind)
        else:
            raise NotImplementedError(k)


def addressed(body, out):
    """Names whose address is taken with & on a plain local (pointer arguments)."""
    def walk(x):
        if isinstance(x, tuple):
            if x and x[0] == "un" and x[1] == "&" and x[2][0] == "name":
                out.add(x[2][1])
            for y in x[1:]:
                walk(y)
        elif isinstance(x, list):
            for y in x:
                walk(y)
    walk(body)


def has_barrier(body):
    found = []

    def walk(x):
        if isinstance(x, tuple):
            if x and x[0] == "call" and x[1] in ("workgroupBarrier", "workgroupUniformLoad"):
                found.append(1)
            for y in x[1:]:
                walk(y)
        elif isinstance(x, list):
            for y in x:
                walk(y)
    walk(body)
    return bool(found)


def compile_module(src, entry_body=None):
    """Compiles WGSL declarations (+ an entry body) to Python; returns the namespace."""
    items = Parser(src).module()
    structs = {it[1]: it[2] for it in items if it[0] == "struct"}
    g = Gen(structs)
    shared_decls = []
    shared_names = {it[3] for it in items if it[0] == "decl" and it[2] == "workgroup"}
    for it in items:
        if it[0] == "fn":
            _, name, params, rt, body = it
            g.boxed = set()
            addressed(body, g.boxed)
            g.boxed -= shared_names              # workgroup variables live in the namespace
            pnames = [p[0] for p in params]
            g.emit(f"def {name}({', '.join(pnames)}):", 0)
            for pn, pt in params:
                if pt[0] != "ptr":
                    g.emit(f"{pn} = arg({pn}, {pt!r})", 1)
            g.stmts(body, 1)
            g.emit("", 0)
        elif it[0] == "decl":
            _, kw, space, name, ty, init = it
            if space == "workgroup":
                shared_decls.append((name, ty))
            else:
                g.boxed = set()
                g.emit(f"{name} = {g.e(init)}", 0)
    if entry_body is not None:
        body = Parser("fn __main() {" + entry_body + "}").module()[0][4]
        g.boxed = set()
        addressed(body, g.boxed)
        g.boxed -= shared_names
        g.emit("def main(lidx, wgi, wid=None, lid=None, gid=None, nwg=None):", 0)
        scalars = [n for n, ty in shared_decls if ty[0] != "array"]
        if scalars:
            g.emit("global " + ", ".join(scalars), 1)
        g.stmts(body, 1)
        if not has_barrier(body):
            g.emit("yield", 1)    # every entry is a generator
    code = "\n".join(g.lines)
    ns = dict(RUNTIME)
    ns["__shared_decls__"] = shared_decls
    exec(compile(code, "<wgsl>", "exec"), ns)
    ns["__source__"] = code
    return ns


# ============================================================================ builtins

def zero(ty):
    name, args = ty
    if name in ("f32",):
        return f32(0)
    if name in ("i32",):
        return i32(0)
    if name in ("u32",):
        return u32(0)
    if name in ("mat3x3f",):
        return Mat(np.zeros((3, 3), f32))
    if name in ("vec3f", "vec4f"):
        return Vec(np.zeros(int(name[3]), f32))
    if name == "array":
        inner, n = args
        count = int(str(n).rstrip("iu"))
        if inner[0] == "atomic":
            dt = {"i32": i32, "u32": u32}[inner[1][0][0]]
            return np.zeros(count, dt)
        return np.zeros(count, {"i32": i32, "u32": u32, "f32": f32}[inner[0]])
    raise NotImplementedError(str(ty))


def arg(v, ty):
    name = ty[0]
    if name == "f32":
        return f32(v)
    if name == "i32":
        return i32(v)
    if name == "u32":
        return u32(v)
    return cp(v)


def _vec(dt, n):
    def make(*xs):
        if not xs:
            return Vec(np.zeros(n, dt))
        parts = []
        for x in xs:
            if isinstance(x, Vec):
                parts.extend(x.a.tolist() if x.a.dtype.kind != "b" else x.a)
            else:
                parts.append(x)
        if len(parts) == 1:
            parts = parts * n
        if dt is f32:
            return Vec(np.array([f32(p) for p in parts], f32))
        if isinstance(xs[0], Vec) and xs[0].a.dtype.kind == "f":   # float -> int conversion truncates
            return Vec(np.array([int(np.trunc(p)) for p in parts]).astype(dt))
        return Vec(np.array([int(p) for p in parts], np.int64).astype(dt))
    return make


def mat3x3f(*xs):
    if not xs:
        return Mat(np.zeros((3, 3), f32))
    if len(xs) == 3:
        return Mat(np.stack([x.a.astype(f32) for x in xs]))
    return Mat(np.array([f32(x) for x in xs], f32).reshape(3, 3))


def _map(fn):
    def g(*xs):
        if isinstance(xs[0], Vec):
            bs = [x.a if isinstance(x, Vec) else np.full(len(xs[0]), x, xs[0].a.dtype) for x in xs]
            return Vec(np.array([fn(*[b[k] for b in bs]) for k in range(len(xs[0]))], dtype=xs[0].a.dtype))
        return fn(*xs)
    return g


def _fmax(a, b):
    if isinstance(a, (np.floating, float)):
        return f32(np.fmax(f32(a), f32(b)))
    return type(a)(max(a, b)) if not isinstance(a, int) else max(a, b)


def _fmin(a, b):
    if isinstance(a, (np.floating, float)):
        return f32(np.fmin(f32(a), f32(b)))
    return type(a)(min(a, b)) if not isinstance(a, int) else min(a, b)


def _clamp(x, lo, hi):
    return _fmin(_fmax(x, lo), hi)


def _dot(a, b):
    x, y = a.a, b.a
    return (x[0] * y[0] + x[1] * y[1]) + x[2] * y[2] if len(x) == 3 else x[0] * y[0] + x[1] * y[1]


def _length(v):
    if not isinstance(v, Vec):
        return f32(abs(v))
    return f32(np.sqrt(_dot(v, v)))


def _normalize(v):
    return v / _length(v)


def _cross(a, b):
    x, y = a.a, b.a
    return Vec(np.array([x[1] * y[2] - x[2] * y[1], x[2] * y[0] - x[0] * y[2], x[0] * y[1] - x[1] * y[0]], f32))


def _transpose(m):
    return Mat(m.c.T.copy())


def _determinant(m):
    c = m.c
    a = c[0, 0] * (c[1, 1] * c[2, 2] - c[2, 1] * c[1, 2])
    b = c[1, 0] * (c[0, 1] * c[2, 2] - c[2, 1] * c[0, 2])
    d = c[2, 0] * (c[0, 1] * c[1, 2] - c[1, 1] * c[0, 2])
    return (a - b) + d


def _select(f, t, cond):
    return t if cond else f


def _any(v):
    return bool(np.any(v.a)) if isinstance(v, Vec) else bool(v)


def _conv(dt):
    def g(x):
        if isinstance(x, Vec):
            return _vec(dt, len(x))(x)
        if dt is f32:
            return f32(x)
        if isinstance(x, (np.floating, float)):
            return dt(int(np.trunc(x)))
        return np.array(x).astype(np.int64).astype(dt)[()] if not isinstance(x, int) else dt(x & 0xFFFFFFFF) \
            if dt is u32 else np.array(x, np.int64).astype(dt)[()]
    return g


def bitcast(ty, x):
    dt = {"u32": u32, "i32": i32, "f32": f32, "vec4i": i32, "vec4f": f32, "vec4u": u32}[ty]
    if isinstance(x, Vec):
        return Vec(x.a.view(dt).copy())
    return np.array([x]).view(dt)[0]


def atomicAdd(buf, idx, v):
    a = buf.arr if isinstance(buf, Buffer) else buf
    old = a[int(idx)]
    a[int(idx)] = old + v
    return old


def atomicMin(buf, idx, v):
    a = buf.arr if isinstance(buf, Buffer) else buf
    old = a[int(idx)]
    a[int(idx)] = min(old, v)
    return old


def atomicMax(buf, idx, v):
    a = buf.arr if isinstance(buf, Buffer) else buf
    old = a[int(idx)]
    a[int(idx)] = max(old, v)
    return old


def atomicLoad(buf, idx):
    a = buf.arr if isinstance(buf, Buffer) else buf
    return a[int(idx)]


def atomicStore(buf, idx, v):
    a = buf.arr if isinstance(buf, Buffer) else buf
    a[int(idx)] = v


RUNTIME = {
    "np": np, "types": types, "f32": f32, "i32": _conv(i32), "u32": _conv(u32), "Vec": Vec, "Mat": Mat,
    "wdiv": wdiv, "wmod": wmod, "cp": cp, "concrete": concrete, "zero": zero, "arg": arg,
    "vec2f": _vec(f32, 2), "vec3f": _vec(f32, 3), "vec4f": _vec(f32, 4), "vec3i": _vec(i32, 3),
    "vec4i": _vec(i32, 4), "vec3u": _vec(u32, 3), "vec4u": _vec(u32, 4), "mat3x3f": mat3x3f,
    "floor": _map(lambda x: f32(np.floor(x))), "round": _map(lambda x: f32(np.rint(x))),
    "abs": _map(lambda x: type(x)(abs(x))), "sqrt": _map(lambda x: f32(np.sqrt(f32(x)))),
    "inverseSqrt": _map(lambda x: f32(f32(1.0) / f32(np.sqrt(f32(x))))),
    "log": _map(lambda x: f32(np.log(f32(x)))), "exp": _map(lambda x: f32(np.exp(f32(x)))),
    "max": _map(_fmax), "min": _map(_fmin), "clamp": _map(_clamp), "dot": _dot, "length": _length,
    "normalize": _normalize, "cross": _cross, "transpose": _transpose, "determinant": _determinant,
    "select": _select, "any": _any, "all": lambda v: bool(np.all(v.a)) if isinstance(v, Vec) else bool(v),
    "sign": _map(lambda x: type(x)(np.sign(x))), "bitcast": bitcast, "atomicAdd": atomicAdd, "atomicMin": atomicMin,
    "atomicMax": atomicMax, "atomicLoad": atomicLoad, "atomicStore": atomicStore,
}
RUNTIME["f32"] = _conv(f32)


# ============================================================================ dispatch

def dispatch(ns, groups, wg, bindings, uniforms):
    """Runs `groups` workgroups of `wg` invocations of ns['main'] with the given bindings. Within a
    workgroup the invocations run in index order up to each barrier, then the next phase."""
    ns["u"] = types.SimpleNamespace(**uniforms)
    ns.update(bindings)
    main = ns["main"]
    for wgi in range(groups):
        for name, ty in ns["__shared_decls__"]:
            ns[name] = zero(ty)
        live = [[main(u32(lidx), u32(wgi)), False] for lidx in range(wg)]
        while any(not x[1] for x in live):
            for x in live:
                if x[1]:
                    continue
                try:
                    next(x[0])
                except StopIteration:
                    x[1] = True


def dispatch3(ns, groups, wg, bindings, uniforms):
    """As dispatch, for a 3-D grid of workgroups of shape wg (local_invocation_index = x + wx (y + wy z))."""
    ns["u"] = types.SimpleNamespace(**uniforms)
    ns.update(bindings)
    main = ns["main"]
    nwg = Vec(np.array(groups, u32))
    size = wg[0] * wg[1] * wg[2]
    for gz in range(groups[2]):
        for gy in range(groups[1]):
            for gx in range(groups[0]):
                for name, ty in ns["__shared_decls__"]:
                    ns[name] = zero(ty)
                wid = np.array([gx, gy, gz], u32)
                live = []
                for li in range(size):
                    lid = np.array([li % wg[0], (li // wg[0]) % wg[1], li // (wg[0] * wg[1])], u32)
                    gid = wid * np.array(wg, u32) + lid
                    live.append([main(u32(li), u32(gx + gy * groups[0]), Vec(wid.copy()), Vec(lid),
                                      Vec(gid), nwg), False])
                while any(not x[1] for x in live):
                    for x in live:
                        if x[1]:
                            continue
                        try:
                            next(x[0])
                        except StopIteration:
                            x[1] = True
