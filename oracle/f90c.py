"""Mechanical Fortran -> C translator for the reference's hot-path modules.

TEST INFRASTRUCTURE ONLY.  No Fortran compiler exists on either machine this project runs on, so
the reference cannot be built.  This script translates the five hot-path modules of the
reference (common/particle.f90, field.f90, sort.f90, boundary_periodic.f90, mom_calc.f90)
statement by statement into one C file, which gcc then compiles (oracle/ref_glue.c, oracle/
reference.py).  Its outputs pin the hand-written restatement in wm_oracle.c: the two must agree
bit for bit on every input (tests/test_reference_pin.py, tests/golden/).

It supports exactly the Fortran subset those files use and stops on anything else:
  modules with SAVE'd module variables; subroutines whose dummies are passed by reference;
  explicit-shape, automatic, allocatable and assumed-shape (1-D) arrays with arbitrary lower
  bounds; array sections and whole-array assignments (elementwise); do / do while / named do with
  exit; if / else if / else; call; allocate; stop (longjmp to the caller); MPI_SENDRECV and
  MPI_ALLREDUCE (single rank: a copy); ieee_set_rounding_mode (restored on return, as the
  Fortran standard requires); the intrinsics dsqrt, sqrt, abs, int, atan, size, and **2.
Typing follows Fortran: default-real literals are C floats, real(8) are doubles, integers are
ints, so mixed expressions promote as in Fortran.  OpenMP directives are comments (serial
semantics).  The generated file goes to oracle/_ref/ (git-ignored); it is never committed.

    python oracle/f90c.py <reference common/ dir> <output .c>
"""
from __future__ import annotations

import re
import sys
from dataclasses import dataclass, field
from pathlib import Path

MODULES = ["boundary_periodic", "particle", "field", "sort", "mom_calc"]


class F90Error(RuntimeError):
    pass


# ------------------------------------------------------------------------ lexing
def logical_lines(text: str) -> list[str]:
    out, buf = [], ""
    for raw in text.splitlines():
        line = raw
        # strip comments (no '!' inside the strings of these files except in write statements)
        q = None
        cut = len(line)
        for i, ch in enumerate(line):
            if q:
                if ch == q:
                    q = None
            elif ch in "'\"":
                q = ch
            elif ch == "!":
                cut = i
                break
        line = line[:cut].rstrip()
        s = line.strip()
        if not s:
            continue
        if buf:
            if s.startswith("&"):
                s = s[1:]
            buf += " " + s
        else:
            buf = s
        if buf.endswith("&"):
            buf = buf[:-1].rstrip()
            continue
        out.append(buf)
        buf = ""
    if buf:
        out.append(buf)
    return out


TOKEN_RE = re.compile(r"""
    (?P<num>(\d+\.\d*|\.\d+|\d+)([de][+-]?\d+)?(_\d+)?)
  | (?P<dot>\.(and|or|not|true|false|eq|ne|lt|le|gt|ge)\.)
  | (?P<name>[a-z_][a-z0-9_]*)
  | (?P<op>\*\*|==|/=|<=|>=|<|>|[-+*/(),:%])
  | (?P<ws>\s+)
""", re.X)


def tokenize(s: str) -> list[tuple[str, str]]:
    toks, i = [], 0
    while i < len(s):
        m = TOKEN_RE.match(s, i)
        if not m:
            raise F90Error(f"cannot tokenize at {s[i:]!r}")
        i = m.end()
        kind = m.lastgroup
        if kind == "ws":
            continue
        toks.append((kind, m.group(0)))
    return toks


def split_top(s: str, sep: str = ",") -> list[str]:
    parts, depth, cur = [], 0, ""
    for ch in s:
        if ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        if ch == sep and depth == 0:
            parts.append(cur.strip())
            cur = ""
        else:
            cur += ch
    if cur.strip():
        parts.append(cur.strip())
    return parts


# ---------------------------------------------------------------------- symbols
@dataclass
class Sym:
    name: str
    typ: str  # 'i', 'd', 'l'
    dims: list = field(default_factory=list)  # [(lb_text, ub_text)], ub_text None for ':'
    kind: str = "local"  # module, dummy, local, save, param, proc
    alloc: bool = False
    assumed: bool = False
    init: str | None = None
    cname: str = ""

    @property
    def rank(self):
        return len(self.dims)


TYPE_RE = re.compile(r"^(integer|real\(8\)|logical)\s*(,.*?)?::\s*(.*)$")


def parse_decl(line: str):
    m = TYPE_RE.match(line)
    if not m:
        return None
    t = {"integer": "i", "real(8)": "d", "logical": "l"}[m.group(1)]
    attrs = [a.strip() for a in split_top(m.group(2)[1:])] if m.group(2) else []
    ents = []
    for e in split_top(m.group(3)):
        init = None
        if "=" in e and not e.startswith("="):
            e, init = [x.strip() for x in e.split("=", 1)]
        mm = re.match(r"^([a-z_][a-z0-9_]*)\s*(\((.*)\))?$", e)
        if not mm:
            raise F90Error(f"bad entity {e!r}")
        dims = []
        if mm.group(3) is not None:
            for dspec in split_top(mm.group(3)):
                if dspec == ":":
                    dims.append((None, None))
                elif ":" in dspec:
                    lb, ub = split_top(dspec, ":")
                    dims.append((lb, ub))
                else:
                    dims.append(("1", dspec))
        ents.append((mm.group(1), dims, init))
    return t, attrs, ents


# ------------------------------------------------------------------ expressions
class Expr:
    def __init__(self, scope, toks, section_vars=None):
        self.scope = scope
        self.toks = toks
        self.i = 0
        self.secvars = section_vars  # per array name: list of loop-var names for section dims

    def peek(self, k=0):
        return self.toks[self.i + k] if self.i + k < len(self.toks) else (None, None)

    def take(self, val=None):
        t = self.peek()
        if val is not None and t[1] != val:
            raise F90Error(f"expected {val!r}, got {t!r} in {' '.join(x[1] for x in self.toks)}")
        self.i += 1
        return t

    def parse(self):
        c, t = self.p_or()
        if self.i != len(self.toks):
            raise F90Error(f"trailing tokens {self.toks[self.i:]}")
        return c, t

    def p_or(self):
        c, t = self.p_and()
        while self.peek()[1] == ".or.":
            self.take()
            c2, _ = self.p_and()
            c, t = f"({c} || {c2})", "l"
        return c, t

    def p_and(self):
        c, t = self.p_not()
        while self.peek()[1] == ".and.":
            self.take()
            c2, _ = self.p_not()
            c, t = f"({c} && {c2})", "l"
        return c, t

    def p_not(self):
        if self.peek()[1] == ".not.":
            self.take()
            c, _ = self.p_not()
            return f"(!{c})", "l"
        return self.p_rel()

    REL = {"==": "==", "/=": "!=", "<": "<", "<=": "<=", ">": ">", ">=": ">=", ".eq.": "==", ".ne.": "!=",
           ".lt.": "<", ".le.": "<=", ".gt.": ">", ".ge.": ">="}

    def p_rel(self):
        c, t = self.p_add()
        if self.peek()[1] in self.REL:
            op = self.REL[self.take()[1]]
            c2, _ = self.p_add()
            return f"({c} {op} {c2})", "l"
        return c, t

    @staticmethod
    def promote(a, b):
        if "d" in (a, b):
            return "d"
        if "f" in (a, b):
            return "f"
        return "i"

    def p_add(self):
        sign = None
        if self.peek()[1] in ("+", "-"):
            sign = self.take()[1]
        c, t = self.p_mul()
        if sign == "-":
            c = f"(-{c})"
        while self.peek()[1] in ("+", "-"):
            op = self.take()[1]
            c2, t2 = self.p_mul()
            c, t = f"({c} {op} {c2})", self.promote(t, t2)
        return c, t

    def p_mul(self):
        c, t = self.p_pow()
        while self.peek()[1] in ("*", "/"):
            op = self.take()[1]
            c2, t2 = self.p_pow()
            c, t = f"({c} {op} {c2})", self.promote(t, t2)
        return c, t

    def p_pow(self):
        c, t = self.p_primary()
        if self.peek()[1] == "**":
            self.take()
            k = self.take()
            if k != ("num", "2"):
                raise F90Error("only **2 is supported")
            fn = {"d": "f90_sqd", "f": "f90_sqf", "i": "f90_sqi"}[t]
            return f"{fn}({c})", t
        return c, t

    def p_primary(self):
        kind, val = self.take()
        if kind == "num":
            return self.number(val)
        if kind == "dot":
            if val == ".true.":
                return "1", "l"
            if val == ".false.":
                return "0", "l"
            raise F90Error(val)
        if val == "(":
            c, t = self.p_or()
            self.take(")")
            return f"({c})", t
        if kind == "name":
            if self.peek()[1] == "(":
                self.take("(")
                args = self.arglist()
                self.take(")")
                return self.call_or_index(val, args)
            return self.scope.ref_scalar(val)
        raise F90Error(f"unexpected token {val!r}")

    def arglist(self):
        """Raw token groups of a parenthesised argument list (top-level commas)."""
        args, cur, depth = [], [], 0
        while True:
            t = self.peek()
            if t[1] is None:
                raise F90Error("unterminated argument list")
            if t[1] == ")" and depth == 0:
                break
            self.take()
            if t[1] == "(":
                depth += 1
            elif t[1] == ")":
                depth -= 1
            if t[1] == "," and depth == 0:
                args.append(cur)
                cur = []
            else:
                cur.append(t)
        if cur:
            args.append(cur)
        return args

    def sub(self, toks):
        e = Expr(self.scope, toks, self.secvars)
        return e.parse()

    INTR = {"dsqrt", "sqrt", "abs", "int", "atan", "size"}

    def call_or_index(self, name, args):
        sym = self.scope.lookup(name)
        if sym is not None and sym.rank > 0:
            return self.scope.element(sym, args, self)
        if name in ("dsqrt", "sqrt"):
            c, _ = self.sub(args[0])
            return f"sqrt((double)({c}))", "d"
        if name == "abs":
            c, t = self.sub(args[0])
            return (f"abs({c})", "i") if t == "i" else (f"fabs({c})", t)
        if name == "int":
            c, _ = self.sub(args[0])
            return f"((int)({c}))", "i"
        if name == "atan":
            c, _ = self.sub(args[0])
            return f"atan({c})", "d"
        if name == "size":
            s = self.scope.lookup(args[0][0][1])
            return self.scope.size_of(s), "i"
        raise F90Error(f"unknown function {name}")

    @staticmethod
    def number(val):
        v = val.split("_")[0]
        if re.fullmatch(r"\d+", v):
            return v, "i"
        if "d" in v:
            return v.replace("d", "e") if re.search(r"d", v) else v, "d"
        # default real: float literal
        if "e" in v:
            m, ex = v.split("e")
            if m.endswith("."):
                m += "0"
            if m.startswith("."):
                m = "0" + m
            return f"{m}e{ex}f", "f"
        if v.endswith("."):
            v += "0"
        if v.startswith("."):
            v = "0" + v
        return f"{v}f", "f"


# ------------------------------------------------------------------------ scopes
class Scope:
    def __init__(self, tr, module, sub=None, parent=None):
        self.tr = tr
        self.module = module
        self.sub = sub
        self.parent = parent
        self.syms: dict[str, Sym] = {}

    def lookup(self, name):
        if name in self.syms:
            return self.syms[name]
        if self.parent:
            return self.parent.lookup(name)
        return None

    def ref_scalar(self, name):
        s = self.lookup(name)
        if s is None:
            raise F90Error(f"unknown name {name}")
        if s.kind == "param":
            return f"({s.cname})", s.typ
        if s.rank > 0:
            raise F90Error(f"array {name} used as scalar")
        if s.kind == "dummy":
            return f"(*{s.cname})", s.typ
        return s.cname, s.typ

    def bound(self, s, k):
        """C expressions (lb, extent) of dimension k of array s."""
        base = s.cname
        return f"{base}__lb{k}", f"{base}__n{k}"

    def size_of(self, s):
        n = " * ".join(f"{s.cname}__n{k}" for k in range(s.rank))
        return f"({n})"

    def data(self, s):
        return s.cname

    def element(self, s, args, ex: Expr):
        if len(args) != s.rank:
            raise F90Error(f"{s.name}: rank {s.rank}, {len(args)} subscripts")
        terms = []
        stride = "1"
        secs = ex.secvars.get(id(args), None) if ex.secvars else None
        for k, a in enumerate(args):
            lb, n = self.bound(s, k)
            if any(t[1] == ":" for t in a):
                if secs is None:
                    raise F90Error(f"section of {s.name} outside an array assignment")
                idx = secs[k]
            else:
                idx, _ = ex.sub(a)
            terms.append(f"(long)(({idx}) - {lb}) * {stride}")
            stride = f"{stride} * {n}" if stride != "1" else n
        return f"{self.data(s)}[{' + '.join(terms)}]", s.typ


# -------------------------------------------------------------------- translator
CTYPE = {"i": "int", "d": "double", "l": "int"}


class Translator:
    def __init__(self):
        self.out: list[str] = []
        self.mod_scopes: dict[str, Scope] = {}
        self.sub_sigs: dict[str, list] = {}  # subroutine name -> list of dummy syms (for calls)
        self.cur_mod = None
        self.labels = 0

    def emit(self, s, ind=0):
        self.out.append("    " * ind + s)

    # ------------------------------------------------------------ modules
    def module(self, name: str, lines: list[str]):
        self.cur_mod = name
        scope = Scope(self, name)
        self.mod_scopes[name] = scope
        self.emit(f"/* ---- module {name} */")
        i = 0
        # header up to 'contains'
        while i < len(lines) and lines[i] != "contains":
            ln = lines[i]
            i += 1
            if ln.startswith(("module ", "use ", "implicit", "private", "public")):
                continue
            d = parse_decl(ln)
            if d is None:
                raise F90Error(f"module {name}: unexpected {ln!r}")
            self.decl_module(scope, *d)
        i += 1
        subs = []
        while i < len(lines):
            ln = lines[i]
            if ln.startswith("subroutine "):
                j, in_iface = i + 1, False
                while in_iface or not re.match(r"^end\s*subroutine", lines[j]):
                    if lines[j] == "interface":
                        in_iface = True
                    elif lines[j] == "end interface":
                        in_iface = False
                    j += 1
                subs.append(lines[i:j + 1])
                i = j + 1
            elif re.match(r"^end\s*module", ln):
                break
            else:
                raise F90Error(f"module {name}: unexpected {ln!r}")
        # prototypes first, then bodies
        for body in subs:
            self.prototype(scope, body[0], body, only_proto=True)
        for body in subs:
            self.subroutine(scope, body)

    def decl_module(self, scope, t, attrs, ents):
        for nm, dims, init in ents:
            s = Sym(nm, t, dims, "module", alloc="allocatable" in attrs, init=init)
            if "parameter" in attrs:
                s.kind = "param"
                s.cname = Expr(scope, tokenize(init)).parse()[0]
                if t == "d":
                    s.cname = f"(double){s.cname}"
            else:
                s.cname = f"{self.cur_mod}__{nm}"
                self.emit_storage(s, static=True)
            scope.syms[nm] = s

    def emit_storage(self, s, static, ind=0):
        st = "static " if static else ""
        ct = CTYPE[s.typ]
        if s.rank == 0:
            init = ""
            if s.init is not None:
                init = " = " + ("1" if s.init == ".true." else "0" if s.init == ".false." else s.init)
            self.emit(f"{st}{ct} {s.cname}{init};", ind)
        else:
            self.emit(f"{st}{ct} *{s.cname};", ind)
            for k in range(s.rank):
                self.emit(f"{st}long {s.cname}__lb{k}, {s.cname}__n{k};", ind)

    # ---------------------------------------------------------- subroutines
    def parse_header(self, line):
        m = re.match(r"^subroutine\s+([a-z_0-9]+)\s*\((.*)\)$", line)
        if not m:
            raise F90Error(line)
        return m.group(1), [a.strip() for a in m.group(2).split(",") if a.strip()]

    def collect(self, mscope, body):
        """Symbols of a subroutine: dummies, locals, procedure dummies; returns (scope, stmts)."""
        name, dummies = self.parse_header(body[0])
        scope = Scope(self, self.cur_mod, name, mscope)
        stmts = []
        i = 1
        procs = set()
        while i < len(body) - 1:
            ln = body[i]
            if ln == "interface":
                j = i + 1
                while body[j] != "end interface":
                    m = re.match(r"^subroutine\s+([a-z_0-9]+)", body[j])
                    if m:
                        procs.add(m.group(1))
                    j += 1
                i = j + 1
                continue
            if ln.startswith("use ") or ln.startswith("use,"):
                i += 1
                continue
            d = parse_decl(ln)
            if d is not None:
                t, attrs, ents = d
                for nm, dims, init in ents:
                    s = Sym(nm, t, dims, init=init, alloc="allocatable" in attrs)
                    if "parameter" in attrs:
                        s.kind = "param"
                        s.cname = Expr(scope, tokenize(init)).parse()[0]
                        if t == "d":
                            s.cname = f"(double){s.cname}"
                    elif nm in dummies:
                        s.kind = "dummy"
                        s.assumed = any(lb is None for lb, _ in dims)
                        s.cname = nm
                    elif "save" in attrs or init is not None:
                        s.kind = "save"
                        s.cname = f"{self.cur_mod}__{name}__{nm}"
                    else:
                        s.kind = "local"
                        s.cname = nm
                    scope.syms[nm] = s
                i += 1
                continue
            stmts.append(ln)
            i += 1
        for p in procs:
            scope.syms[p] = Sym(p, "i", [], "proc", cname=p)
        return name, dummies, scope, stmts

    def prototype(self, mscope, header, body, only_proto=False):
        name, dummies, scope, _ = self.collect(mscope, body)
        params = []
        for d in dummies:
            s = scope.syms[d]
            if s.kind == "proc":
                params.append(f"void (*{d})()")
            elif s.assumed:
                params.append(f"{CTYPE[s.typ]} *{d}")
                params.append(f"long {d}__size")
            else:
                params.append(f"{CTYPE[s.typ]} *{d}")
        self.sub_sigs[name] = (dummies, scope)
        self.emit(f"void ref_{name}({', '.join(params)});")

    def subroutine(self, mscope, body):
        name, dummies, scope, stmts = self.collect(mscope, body)
        uses_round = any("ieee_set_rounding_mode" in s for s in stmts)
        # storage for SAVE'd locals at file scope
        for s in scope.syms.values():
            if s.kind == "save":
                self.emit_storage(s, static=False)
        params = []
        for d in dummies:
            s = scope.syms[d]
            if s.kind == "proc":
                params.append(f"void (*{d})()")
            elif s.assumed:
                params.append(f"{CTYPE[s.typ]} *{d}")
                params.append(f"long {d}__size")
            else:
                params.append(f"{CTYPE[s.typ]} *{d}")
        self.emit(f"void ref_{name}({', '.join(params)})")
        self.emit("{")
        if uses_round:
            self.emit("const int f90_round_save = fegetround();", 1)
        # bounds of dummy arrays, then locals
        for d in dummies:
            s = scope.syms[d]
            if s.kind == "dummy" and s.rank > 0:
                if s.assumed:
                    self.emit(f"const long {s.cname}__lb0 = 1, {s.cname}__n0 = {s.cname}__size;", 1)
                else:
                    self.bounds_decl(scope, s, 1)
        frees = []
        for s in scope.syms.values():
            if s.kind == "local":
                if s.rank == 0:
                    self.emit(f"{CTYPE[s.typ]} {s.cname} = 0;", 1)
                elif s.alloc:
                    raise F90Error("local allocatable without save")
                else:
                    self.bounds_decl(scope, s, 1)
                    n = " * ".join(f"{s.cname}__n{k}" for k in range(s.rank))
                    self.emit(f"{CTYPE[s.typ]} *{s.cname} = ({CTYPE[s.typ]} *)calloc((size_t)({n}) + 1, sizeof({CTYPE[s.typ]}));", 1)
                    frees.append(s.cname)
        self.block(scope, stmts, 1)
        self.emit("f90_return:;", 1)
        for f in frees:
            self.emit(f"free({f});", 1)
        if uses_round:
            self.emit("fesetround(f90_round_save);", 1)
        self.emit("}")
        self.emit("")

    def bounds_decl(self, scope, s, ind):
        for k, (lb, ub) in enumerate(s.dims):
            lbc, _ = Expr(scope, tokenize(lb)).parse()
            ubc, _ = Expr(scope, tokenize(ub)).parse()
            self.emit(f"const long {s.cname}__lb{k} = {lbc}, {s.cname}__n{k} = ({ubc}) - ({lbc}) + 1;", ind)

    # ------------------------------------------------------------ statements
    def block(self, scope, stmts, ind):
        i = 0
        stack = []
        for ln in stmts:
            self.statement(scope, ln, ind + len(stack), stack)
        if stack:
            raise F90Error(f"unclosed blocks {stack}")

    def cond(self, scope, text):
        c, _ = Expr(scope, tokenize(text)).parse()
        return c

    def statement(self, scope, ln, ind, stack):
        m = re.match(r"^if\s*\((.*)\)\s*then$", ln)
        if m and self.balanced(m.group(1)):
            self.emit(f"if ({self.cond(scope, m.group(1))}) {{", ind)
            stack.append("if")
            return
        m = re.match(r"^else\s*if\s*\((.*)\)\s*then$", ln)
        if m:
            self.emit(f"}} else if ({self.cond(scope, m.group(1))}) {{", ind - 1)
            return
        if ln == "else":
            self.emit("} else {", ind - 1)
            return
        if re.match(r"^end\s*if$", ln):
            stack.pop()
            self.emit("}", ind - 1)
            return
        # select case on an integer: an if / else-if chain over the case value lists
        m = re.match(r"^select\s+case\s*\((.*)\)$", ln)
        if m:
            self.labels += 1
            sel = f"f90_sel{self.labels}"
            self.emit(f"{{ const long {sel} = {self.cond(scope, m.group(1))};", ind)
            self.emit("if (0) {", ind)
            stack.append(("select", sel))
            return
        m = re.match(r"^case\s*\((.*)\)$", ln)
        if m and stack and isinstance(stack[-1], tuple) and stack[-1][0] == "select":
            sel = stack[-1][1]
            vals = [Expr(scope, tokenize(v)).parse()[0] for v in split_top(m.group(1))]
            self.emit("} else if (" + " || ".join(f"{sel} == ({v})" for v in vals) + ") {", ind - 1)
            return
        if re.match(r"^case\s+default$", ln) and stack and isinstance(stack[-1], tuple) and stack[-1][0] == "select":
            self.emit("} else {", ind - 1)
            return
        if re.match(r"^end\s*select$", ln):
            stack.pop()
            self.emit("} }", ind - 1)
            return
        m = re.match(r"^(?:([a-z_0-9]+)\s*:\s*)?do\s+while\s*\((.*)\)$", ln)
        if m:
            self.emit(f"while ({self.cond(scope, m.group(2))}) {{", ind)
            stack.append(("do", m.group(1)))
            return
        m = re.match(r"^(?:([a-z_0-9]+)\s*:\s*)?do\s+([a-z_0-9]+)\s*=\s*(.*)$", ln)
        if m:
            label, var, rng = m.groups()
            parts = split_top(rng)
            if len(parts) != 2:
                raise F90Error(f"do with step: {ln}")
            lo = Expr(scope, tokenize(parts[0])).parse()[0]
            hi = Expr(scope, tokenize(parts[1])).parse()[0]
            vc, _ = scope.ref_scalar(var)
            self.labels += 1
            hv = f"f90_hi{self.labels}"
            self.emit(f"{{ const long {hv} = {hi};", ind)
            self.emit(f"for ({vc} = {lo}; {vc} <= {hv}; {vc}++) {{", ind)
            stack.append(("for", label))
            return
        if re.match(r"^end\s*do(\s+[a-z_0-9]+)?$", ln):
            kind, label = stack.pop()
            self.emit("}" + (" }" if kind == "for" else ""), ind - 1)
            if label:
                self.emit(f"{label}_exit:;", ind - 1)
            return
        m = re.match(r"^exit\s*([a-z_0-9]*)$", ln)
        if m:
            self.emit(f"goto {m.group(1)}_exit;" if m.group(1) else "break;", ind)
            return
        m = re.match(r"^if\s*\((.*)\)\s*(.+)$", ln)
        if m:
            # single-line if: split at the matching parenthesis
            depth, k = 0, 0
            for k, ch in enumerate(ln):
                if ch == "(":
                    depth += 1
                elif ch == ")":
                    depth -= 1
                    if depth == 0:
                        break
            condt = ln[ln.index("(") + 1:k]
            rest = ln[k + 1:].strip()
            self.emit(f"if ({self.cond(scope, condt)}) {{", ind)
            self.statement(scope, rest, ind + 1, stack)
            self.emit("}", ind)
            return
        if ln.startswith("write"):
            return
        if ln == "stop":
            self.emit("f90_stop();", ind)
            return
        if ln.startswith("allocate"):
            inner = ln[ln.index("(") + 1:ln.rindex(")")]
            for item in split_top(inner):
                mm = re.match(r"^([a-z_0-9]+)\s*\((.*)\)$", item)
                s = scope.lookup(mm.group(1))
                dims = []
                for dspec in split_top(mm.group(2)):
                    if ":" in dspec:
                        dims.append(split_top(dspec, ":"))
                    else:
                        dims.append(["1", dspec])
                tot = []
                for k, (lb, ub) in enumerate(dims):
                    lbc = Expr(scope, tokenize(lb)).parse()[0]
                    ubc = Expr(scope, tokenize(ub)).parse()[0]
                    self.emit(f"{s.cname}__lb{k} = {lbc}; {s.cname}__n{k} = ({ubc}) - ({lbc}) + 1;", ind)
                    tot.append(f"{s.cname}__n{k}")
                self.emit(f"{s.cname} = ({CTYPE[s.typ]} *)calloc((size_t)({' * '.join(tot)}) + 1, sizeof({CTYPE[s.typ]}));", ind)
            return
        m = re.match(r"^call\s+([a-z_0-9]+)\s*\((.*)\)$", ln)
        if m:
            self.call(scope, m.group(1), m.group(2), ind)
            return
        # assignment
        k = self.assign_split(ln)
        if k is None:
            raise F90Error(f"unsupported statement: {ln}")
        self.assignment(scope, ln[:k].strip(), ln[k + 1:].strip(), ind)

    @staticmethod
    def balanced(s):
        d = 0
        for ch in s:
            d += ch == "("
            d -= ch == ")"
            if d < 0:
                return False
        return d == 0

    @staticmethod
    def assign_split(ln):
        depth = 0
        for k, ch in enumerate(ln):
            if ch == "(":
                depth += 1
            elif ch == ")":
                depth -= 1
            elif ch == "=" and depth == 0:
                prev = ln[k - 1] if k else ""
                nxt = ln[k + 1] if k + 1 < len(ln) else ""
                if prev not in "<>/=" and nxt != "=":
                    return k
        return None

    # ------------------------------------------------------------ assignment
    def assignment(self, scope, lhs, rhs, ind):
        ltoks = tokenize(lhs)
        name = ltoks[0][1]
        s = scope.lookup(name)
        if s is None:
            raise F90Error(f"assignment to unknown {name}")
        sections = s.rank > 0 and (len(ltoks) == 1 or any(t[1] == ":" for t in ltoks))
        if not sections:
            lc, _ = Expr(scope, ltoks).parse() if len(ltoks) > 1 else scope.ref_scalar(name)
            rc, _ = Expr(scope, tokenize(rhs)).parse()
            self.emit(f"{lc} = {rc};", ind)
            return
        # elementwise loops over the section dimensions of the left-hand side
        lsub = self.subscripts(ltoks, s)
        loopdims = [k for k, a in enumerate(lsub) if a is None or any(t[1] == ":" for t in a)]
        self.labels += 1
        tag = self.labels
        ranges = []
        for n, k in enumerate(loopdims):
            lo, hi = self.section_range(scope, s, k, lsub[k])
            ranges.append((f"f90_t{tag}_{n}", lo, hi))
        for var, lo, hi in reversed(ranges):
            self.emit(f"for (long {var} = 0; {var} <= ({hi}) - ({lo}); {var}++) {{", ind)
            ind += 1
        lc = self.section_ref(scope, s, lsub, [(v, lo) for v, lo, hi in ranges])
        rc = self.section_expr(scope, rhs, [(v, None) for v, lo, hi in ranges])
        self.emit(f"{lc} = {rc};", ind)
        for _ in ranges:
            ind -= 1
            self.emit("}", ind)

    @staticmethod
    def subscripts(toks, s):
        if len(toks) == 1:
            return [None] * s.rank
        e = Expr(None, toks[2:])
        args = e.arglist()
        return args

    def section_range(self, scope, s, k, arg):
        lb, n = scope.bound(s, k)
        if arg is None or (len(arg) == 1 and arg[0][1] == ":"):
            return lb, f"{lb} + {n} - 1"
        parts, cur = [], []
        for t in arg:
            if t[1] == ":":
                parts.append(cur)
                cur = []
            else:
                cur.append(t)
        parts.append(cur)
        lo = Expr(scope, parts[0]).parse()[0] if parts[0] else lb
        hi = Expr(scope, parts[1]).parse()[0] if parts[1] else f"{lb} + {n} - 1"
        return lo, hi

    def section_ref(self, scope, s, sub, loopvars):
        terms = []
        stride = "1"
        li = 0
        for k in range(s.rank):
            lb, n = scope.bound(s, k)
            a = sub[k]
            if a is None or any(t[1] == ":" for t in a):
                lo, _ = self.section_range(scope, s, k, a)
                idx = f"({lo}) + {loopvars[li][0]}"
                li += 1
            else:
                idx = Expr(scope, a).parse()[0]
            terms.append(f"(long)(({idx}) - {lb}) * {stride}")
            stride = f"{stride} * {n}" if stride != "1" else n
        return f"{s.cname}[{' + '.join(terms)}]"

    def section_expr(self, scope, rhs, loopvars):
        """Translate an array-valued expression: array names / sections take the loop indices."""
        toks = tokenize(rhs)
        out = []
        i = 0
        pieces = []
        while i < len(toks):
            kind, val = toks[i]
            s = scope.lookup(val) if kind == "name" else None
            if s is not None and s.rank > 0:
                if i + 1 < len(toks) and toks[i + 1][1] == "(":
                    depth, j = 0, i + 1
                    while True:
                        if toks[j][1] == "(":
                            depth += 1
                        elif toks[j][1] == ")":
                            depth -= 1
                            if depth == 0:
                                break
                        j += 1
                    sub = Expr(None, toks[i + 2:j + 1]).arglist()
                    i = j + 1
                else:
                    sub = [None] * s.rank
                    i += 1
                ref = self.section_ref(scope, s, sub, loopvars) if any(
                    a is None or any(t[1] == ":" for t in a) for a in sub) else None
                if ref is None:
                    ref = Expr(scope, [(kind, val), ("op", "(")] + [t for a in self._join(sub) for t in a] + [("op", ")")]).parse()[0]
                pieces.append(("name", f"f90_ref{len(out)}"))
                out.append((f"f90_ref{len(out)}", ref, s.typ))
            else:
                pieces.append(toks[i])
                i += 1
        # parse the rebuilt expression with placeholders standing for the array elements
        ph = Scope(self, scope.module, scope.sub, scope)
        for nm, ref, typ in out:
            ph.syms[nm] = Sym(nm, typ, [], "local", cname=f"({ref})")
        c, _ = Expr(ph, pieces).parse()
        return c

    @staticmethod
    def _join(sub):
        res = []
        for n, a in enumerate(sub):
            if n:
                res.append([("op", ",")])
            res.append(a)
        return res

    # ------------------------------------------------------------------ calls
    def call(self, scope, name, argtext, ind):
        args = split_top(argtext) if argtext.strip() else []
        if name == "ieee_set_rounding_mode":
            if args != ["ieee_down"]:
                raise F90Error(args)
            self.emit("fesetround(FE_DOWNWARD);", ind)
            return
        if name in ("mpi_sendrecv", "mpi_allreduce"):
            cargs = [self.actual(scope, a) for a in args]
            self.emit(f"f90_{name}({', '.join(cargs)});", ind)
            return
        s = scope.lookup(name)
        if s is not None and s.kind == "proc":
            cargs = [self.actual(scope, a) for a in args]
            self.emit(f"{name}({', '.join(cargs)});", ind)
            return
        if name not in self.sub_sigs:
            raise F90Error(f"call to unknown {name}")
        dummies, dscope = self.sub_sigs[name]
        cargs = []
        for a, d in zip(args, dummies):
            ds = dscope.syms[d]
            cargs.append(self.actual(scope, a))
            if ds.assumed:
                s2 = scope.lookup(a)
                cargs.append(scope.size_of(s2))
        self.emit(f"ref_{name}({', '.join(cargs)});", ind)

    def actual(self, scope, a):
        """Fortran passes by reference: an address for every actual argument."""
        toks = tokenize(a)
        if len(toks) == 1 and toks[0][0] == "name":
            s = scope.lookup(toks[0][1])
            if s is not None:
                if s.kind == "proc":
                    return f"(void (*)())ref_{s.name}" if s.name in self.sub_sigs else s.name
                if s.rank > 0:
                    return s.cname
                if s.kind == "dummy":
                    return s.cname
                if s.kind != "param":
                    return f"&{s.cname}"
            elif toks[0][1] in self.sub_sigs:
                return f"(void (*)())ref_{toks[0][1]}"
        if len(toks) > 1 and toks[0][0] == "name" and toks[1][1] == "(":
            s = scope.lookup(toks[0][1])
            if s is not None and s.rank > 0:
                c, _ = Expr(scope, toks).parse()
                return f"&{c}"
        c, t = Expr(scope, toks).parse()
        return f"(({CTYPE[t]}[]){{{c}}})"


PRELUDE = r"""/* Generated by oracle/f90c.py from the reference common/ modules; not committed. */
#include <fenv.h>
#include <math.h>
#include <setjmp.h>
#include <stdlib.h>
#include <string.h>
#include "ref_runtime.h"
static inline double f90_sqd(double x) { return x * x; }
static inline float f90_sqf(float x) { return x * x; }
static inline int f90_sqi(int x) { return x * x; }
"""


def translate(common_dir: Path, extra=()) -> str:
    """common/ modules, then extra module files (the applications' boundary modules), each
    named after its file."""
    tr = Translator()
    tr.out.append(PRELUDE)
    for mod in MODULES:
        text = (common_dir / f"{mod}.f90").read_text().lower()
        tr.module(mod, logical_lines(text))
    for path in extra:
        tr.module(Path(path).stem, logical_lines(Path(path).read_text().lower()))
    return "\n".join(tr.out) + "\n"


def main(argv):
    src = Path(argv[1])
    dst = Path(argv[2])
    dst.parent.mkdir(parents=True, exist_ok=True)
    dst.write_text(translate(src))


if __name__ == "__main__":
    main(sys.argv)
