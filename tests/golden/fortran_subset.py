"""A translator from the Fortran 90 subset of PixelFlow's OpenMP programs to
Python, used only to generate golden vectors (test infrastructure; no
product code imports it).

It executes the reference's own source text -- the main program and the
subroutines of the step, with gfortran's semantics for the plain FP64 build
(-fdefault-real-8: every `real`, and every real literal, is an IEEE double)
-- so that the C oracle can be checked against the reference itself on small
grids, where no Fortran compiler is available.  Supported: modules with
parameters and variables, `contains`, subroutines with by-reference
arguments (arrays passed as objects; scalars copied in and out), `real`,
`integer`, `logical`, `character` declarations with `dimension` bounds,
`do` loops with steps, block and one-line `if`, `call`, assignment,
`return`, `exit`, `cycle`, list-directed `read` from files opened with
`open`, namelist `read`s (the caller supplies the group's values in
`Program.nml_values`), and the intrinsics the programs use.  `!$omp`
directives are comments (the parallel loops are order-independent, as the
reference requires).  `write` records its values, unformatted, one list per
record in `Program.writes[unit]` (an internal write into a character
variable under "internal", the variable left unchanged); `print` and
`close` are ignored.  Expressions are
evaluated left to right as written, one IEEE operation per Fortran operator
(no fused multiply-add), `x**2` as `x*x`, integer `/` truncating toward zero,
`mod` with the sign of its first argument.

Arrays are flat Python lists indexed column-major with their declared lower
bounds, as Fortran stores them.  Parameters (such as the static array sizes
md, nd) may be overridden by the caller; they size storage only.
"""
from __future__ import annotations

import math
import re
from typing import Dict, List, Optional, Tuple

# ---------------------------------------------------------------- source ----


def _strip_comment(line: str) -> str:
    out, q = [], None
    for ch in line:
        if q:
            out.append(ch)
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
            out.append(ch)
        elif ch == "!":
            break
        else:
            out.append(ch)
    return "".join(out)


def logical_lines(text: str) -> List[str]:
    """Free-form source -> statements: comments removed, `&` continuations
    joined, lower case outside strings, `;` separated statements split."""
    out, cur = [], ""
    for raw in text.splitlines():
        line = _strip_comment(raw).rstrip()
        if not line.strip():
            continue
        s = line.strip()
        if cur and s.startswith("&"):
            s = s[1:]
        if s.endswith("&"):
            cur += s[:-1] + " "
            continue
        cur += s
        out.append(cur)
        cur = ""
    res = []
    for st in out:
        low = _lower_outside_strings(st)
        res.extend(x.strip() for x in low.split(";") if x.strip())
    return res


def _lower_outside_strings(s: str) -> str:
    out, q = [], None
    for ch in s:
        if q:
            out.append(ch)
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
            out.append(ch)
        else:
            out.append(ch.lower())
    return "".join(out)


# ------------------------------------------------------------ expressions ----

_TOKEN = re.compile(r"""
    (?P<num>(\d+\.\d*|\.\d+|\d+)([eEdD][+-]?\d+)?)
  | (?P<dotop>\.(and|or|not|eq|ne|lt|le|gt|ge|true|false|eqv|neqv)\.)
  | (?P<name>[a-z_][a-z_0-9]*)
  | (?P<str>'[^']*'|"[^"]*")
  | (?P<op>\*\*|//|==|/=|<=|>=|[-+*/(),<>=:])
  | (?P<ws>\s+)
""", re.X)


def tokenize(s: str) -> List[Tuple[str, str]]:
    pos, out = 0, []
    while pos < len(s):
        m = _TOKEN.match(s, pos)
        if not m:
            raise SyntaxError(f"cannot tokenize {s[pos:]!r} in {s!r}")
        pos = m.end()
        kind = m.lastgroup
        if kind == "ws":
            continue
        out.append((kind, m.group(kind)))
    return out


class Expr:
    """Recursive-descent translation of one expression to Python source.
    `types` maps names to ('int'|'real'|'logical'|'char', is_array)."""

    def __init__(self, toks, ctx):
        self.t = toks
        self.i = 0
        self.ctx = ctx

    def peek(self, k=0):
        return self.t[self.i + k] if self.i + k < len(self.t) else (None, None)

    def take(self):
        tok = self.t[self.i]
        self.i += 1
        return tok

    def expect(self, v):
        k, x = self.take()
        if x != v:
            raise SyntaxError(f"expected {v!r}, got {x!r}")

    # each parse_* returns (python_source, type) with type 'int' | 'real' | 'logical' | 'char'
    def parse(self):
        return self.p_eqv()

    def p_eqv(self):
        a, ta = self.p_or()
        while self.peek()[1] in (".eqv.", ".neqv."):
            op = self.take()[1]
            b, _ = self.p_or()
            a, ta = (f"({a} == {b})" if op == ".eqv." else f"({a} != {b})"), "logical"
        return a, ta

    def p_or(self):
        a, ta = self.p_and()
        while self.peek()[1] == ".or.":
            self.take()
            b, _ = self.p_and()
            a, ta = f"({a} or {b})", "logical"
        return a, ta

    def p_and(self):
        a, ta = self.p_not()
        while self.peek()[1] == ".and.":
            self.take()
            b, _ = self.p_not()
            a, ta = f"({a} and {b})", "logical"
        return a, ta

    def p_not(self):
        if self.peek()[1] == ".not.":
            self.take()
            a, _ = self.p_not()
            return f"(not {a})", "logical"
        return self.p_rel()

    _REL = {"==": "==", ".eq.": "==", "/=": "!=", ".ne.": "!=", "<": "<", ".lt.": "<", "<=": "<=",
            ".le.": "<=", ">": ">", ".gt.": ">", ">=": ">=", ".ge.": ">="}

    def p_rel(self):
        a, ta = self.p_concat()
        if self.peek()[1] in self._REL:
            op = self._REL[self.take()[1]]
            b, tb = self.p_concat()
            return f"({a} {op} {b})", "logical"
        return a, ta

    def p_concat(self):
        a, ta = self.p_add()
        while self.peek()[1] == "//":
            self.take()
            b, _ = self.p_add()
            a, ta = f"({a} + {b})", "char"
        return a, ta

    def p_add(self):
        # a leading sign applies to the first term (Fortran: -a*b is -(a*b))
        sign = None
        if self.peek()[1] in ("+", "-"):
            sign = self.take()[1]
        a, ta = self.p_mul()
        if sign == "-":
            a = f"(-{a})"
        while self.peek()[1] in ("+", "-"):
            op = self.take()[1]
            b, tb = self.p_mul()
            a, ta = f"({a} {op} {b})", _num(ta, tb)
        return a, ta

    def p_mul(self):
        a, ta = self.p_pow()
        while self.peek()[1] in ("*", "/"):
            op = self.take()[1]
            b, tb = self.p_pow()
            if op == "/" and ta == "int" and tb == "int":
                a, ta = f"_idiv({a}, {b})", "int"
            else:
                a, ta = f"({a} {op} {b})", _num(ta, tb)
        return a, ta

    def p_pow(self):
        a, ta = self.p_unary()
        if self.peek()[1] == "**":
            self.take()
            b, tb = self.p_pow()  # right associative
            if b == "2" and tb == "int":
                return f"_sq({a})", ta
            if tb == "int" and ta == "int":
                return f"({a} ** {b})", "int"
            return f"_pow({a}, {b})", "real"
        return a, ta

    def p_unary(self):
        if self.peek()[1] in ("+", "-"):
            op = self.take()[1]
            a, ta = self.p_pow()
            return (f"(-{a})" if op == "-" else a), ta
        return self.p_primary()

    def p_primary(self):
        kind, v = self.take()
        if kind == "num":
            if re.fullmatch(r"\d+", v):
                return v, "int"
            return repr(float(v.replace("d", "e"))), "real"
        if kind == "dotop" and v in (".true.", ".false."):
            return ("True" if v == ".true." else "False"), "logical"
        if kind == "str":
            return repr(v[1:-1]), "char"
        if v == "(":
            a, ta = self.parse()
            self.expect(")")
            return f"({a})", ta
        if kind == "name":
            if self.peek()[1] == "(":
                self.take()
                args = []
                if self.peek()[1] != ")":
                    while True:
                        args.append(self.parse())
                        if self.peek()[1] == ",":
                            self.take()
                            continue
                        break
                self.expect(")")
                return self.ctx.ref(v, args)
            return self.ctx.var(v)
        raise SyntaxError(f"unexpected token {v!r}")


def _num(a, b):
    return "real" if "real" in (a, b) else "int"


# ------------------------------------------------------------- runtime ----

def _idiv(a, b):
    q = abs(a) // abs(b)
    return q if (a >= 0) == (b >= 0) else -q


def _mod(a, b):
    if isinstance(a, int) and isinstance(b, int):
        return a - _idiv(a, b) * b
    return math.fmod(a, b)


def _sq(x):
    return x * x


def _pow(a, b):
    return float(a) ** b


def _max(*xs):
    r = xs[0]
    for x in xs[1:]:
        if x > r:
            r = x
    return float(r) if any(isinstance(x, float) for x in xs) else r


def _min(*xs):
    r = xs[0]
    for x in xs[1:]:
        if x < r:
            r = x
    return float(r) if any(isinstance(x, float) for x in xs) else r


INTRINSICS = {
    "max": ("_max", None), "min": ("_min", None), "abs": ("abs", "same"), "mod": ("_mod", "same"),
    "sqrt": ("math.sqrt", "real"), "cos": ("math.cos", "real"), "sin": ("math.sin", "real"),
    "atan": ("math.atan", "real"), "exp": ("math.exp", "real"), "tanh": ("math.tanh", "real"),
    "real": ("float", "real"), "dble": ("float", "real"), "float": ("float", "real"), "int": ("int", "int"),
    "nint": ("round", "int"), "trim": ("_trim", "char"),
}


def _trim(s):
    return s.rstrip()


class Array:
    """A Fortran array: flat column-major storage with lower bounds."""

    def __init__(self, bounds: List[Tuple[int, int]], kind: str):
        self.lo = [b[0] for b in bounds]
        self.ext = [b[1] - b[0] + 1 for b in bounds]
        n = 1
        for e in self.ext:
            n *= e
        zero = 0.0 if kind == "real" else (0 if kind == "int" else False)
        self.data = [zero] * n
        self.strides = []
        s = 1
        for e in self.ext:
            self.strides.append(s)
            s *= e
        # flat offset = sum((i_d - lo_d) * stride_d) = sum(i_d * stride_d) - base
        self.base = sum(l * st for l, st in zip(self.lo, self.strides))


# ------------------------------------------------------------ translator ----

class Unit:
    def __init__(self, kind, name, args=None):
        self.kind = kind      # 'module' | 'program' | 'subroutine'
        self.name = name
        self.args = args or []
        self.body: List[str] = []
        self.uses: List[str] = []
        self.contains: List["Unit"] = []


def split_units(lines: List[str]) -> List[Unit]:
    units, stack = [], []
    for ln in lines:
        m = re.match(r"(module|program)\s+(\w+)$", ln)
        if m and not ln.startswith("module procedure"):
            u = Unit(m.group(1), m.group(2))
            (stack[-1].contains if stack else units).append(u)
            stack.append(u)
            continue
        m = re.match(r"subroutine\s+(\w+)\s*(\((.*)\))?$", ln)
        if m:
            args = [a.strip() for a in (m.group(3) or "").split(",") if a.strip()]
            u = Unit("subroutine", m.group(1), args)
            (stack[-1].contains if stack else units).append(u)
            stack.append(u)
            continue
        if re.match(r"end\s*(module|program|subroutine)\b", ln) or (ln == "end" and stack):
            stack.pop()
            continue
        if ln == "contains":
            continue
        if not stack:
            continue
        stack[-1].body.append(ln)
    return units


_DECL = re.compile(r"^(real|integer|logical|character|double\s+precision)\b(.*)$")


class Context:
    """Name resolution while translating one unit."""

    def __init__(self, prog: "Program", unit: Unit):
        self.prog = prog
        self.unit = unit
        self.local: Dict[str, dict] = {}   # name -> {kind, dims, param, value}

    def lookup(self, name):
        if name in self.local:
            return self.local[name], "local"
        for mod in self.unit.uses:
            if name in self.prog.modvars.get(mod, {}):
                return self.prog.modvars[mod][name], mod
        return None, None

    def var(self, name):
        info, where = self.lookup(name)
        if info is None:
            raise NameError(f"{self.unit.name}: unknown name {name}")
        if info.get("param"):
            v = info["value"]
            return repr(v), info["kind"]
        if where == "local":
            return f"L_{name}", info["kind"]
        return f"M[{where!r}][{name!r}]", info["kind"]

    def ref(self, name, args):
        info, where = self.lookup(name)
        if info is not None and info.get("dims"):
            arr = f"L_{name}" if where == "local" else f"M[{where!r}][{name!r}]"
            idx = " + ".join(f"({a[0]})*{arr}.strides[{d}]" for d, a in enumerate(args))
            return f"{arr}.data[{idx} - {arr}.base]", info["kind"]
        if name in INTRINSICS:
            fn, rk = INTRINSICS[name]
            srcs = ", ".join(a[0] for a in args)
            if rk is None:
                rk = "real" if any(a[1] == "real" for a in args) else "int"
            elif rk == "same":
                rk = args[0][1]
            return f"{fn}({srcs})", rk
        raise NameError(f"{self.unit.name}: unknown function or array {name}")

    def expr(self, s):
        return Expr(tokenize(s), self).parse()


class Program:
    """Translate a set of Fortran sources; run the main program."""

    def __init__(self, sources: List[str], overrides: Optional[Dict[str, object]] = None,
                 stubs: Optional[Dict[str, object]] = None):
        self.overrides = overrides or {}
        self.stubs = stubs or {}
        lines = []
        for s in sources:
            lines.extend(logical_lines(s))
        self.units = split_units(lines)
        self.modvars: Dict[str, Dict[str, dict]] = {}
        self.subs: Dict[str, Unit] = {}
        self.main: Optional[Unit] = None
        for u in self.units:
            self._collect(u)
        self.M: Dict[str, Dict[str, object]] = {}
        self.files: Dict[int, List[str]] = {}
        self.writes: Dict[object, List[list]] = {}
        self.vfs: Dict[str, str] = {}
        self.compiled = {}
        for m in [u for u in self._walk() if u.kind == "module"]:
            self._module(m)

    def _walk(self):
        stack = list(self.units)
        while stack:
            u = stack.pop(0)
            yield u
            stack.extend(u.contains)

    def _collect(self, u):
        if u.kind == "program":
            self.main = u
        if u.kind == "subroutine":
            self.subs[u.name] = u
        for c in u.contains:
            if c.kind == "subroutine":
                c.uses.append(u.name)  # host association of module variables
            self._collect(c)

    # declarations ---------------------------------------------------------
    def _decl(self, ctx: Context, ln: str):
        m = _DECL.match(ln)
        if not m:
            return False
        kind = {"real": "real", "integer": "int", "logical": "logical", "character": "char",
                "double precision": "real"}[re.sub(r"\s+", " ", m.group(1))]
        rest = m.group(2)
        if "::" in rest:
            attrs, names = rest.split("::", 1)
        else:
            attrs, names = "", rest
        attrs = attrs.strip().lstrip(",")
        param = "parameter" in attrs
        dims = None
        dm = re.search(r"dimension\s*\((.*)\)", attrs)
        if dm:
            dims = self._split_top(dm.group(1))
        for item in self._split_top(names):
            item = item.strip()
            if not item:
                continue
            val = None
            if "=" in item and not item.startswith("="):
                item, val = [x.strip() for x in item.split("=", 1)]
            im = re.match(r"(\w+)\s*(\((.*)\))?$", item)
            nm = im.group(1)
            ddims = self._split_top(im.group(3)) if im.group(3) else dims
            info = {"kind": kind, "dims": ddims}
            if param:
                info["param"] = True
                if nm in self.overrides:
                    info["value"] = self.overrides[nm]
                else:
                    src, t = ctx.expr(val)
                    v = eval(src, {"math": math, "_max": _max, "_min": _min, "_sq": _sq, "_pow": _pow,
                                   "_idiv": _idiv, "_mod": _mod})
                    info["value"] = float(v) if kind == "real" else v
            ctx.local[nm] = info
        return True

    @staticmethod
    def _split_top(s):
        out, depth, cur, quote = [], 0, "", None
        for ch in s:
            if quote:
                quote = None if ch == quote else quote
            elif ch in "'\"":
                quote = ch
            elif ch == "(":
                depth += 1
            elif ch == ")":
                depth -= 1
            if ch == "," and depth == 0 and not quote:
                out.append(cur)
                cur = ""
            else:
                cur += ch
        if cur.strip():
            out.append(cur)
        return [x.strip() for x in out]

    def _bounds_src(self, ctx, dims):
        parts = []
        for d in dims:
            if ":" in d:
                lo, hi = d.split(":", 1)
            else:
                lo, hi = "1", d
            parts.append(f"({ctx.expr(lo)[0]}, {ctx.expr(hi)[0]})")
        return "[" + ", ".join(parts) + "]"

    def _module(self, m: Unit):
        ctx = Context(self, m)
        m.uses = [ln.split()[1].rstrip(",") for ln in m.body if ln.startswith("use ")]
        for ln in m.body:
            if ln.startswith(("use ", "implicit")):
                continue
            if ln.startswith("namelist"):
                continue
            if not self._decl(ctx, ln):
                raise SyntaxError(f"module {m.name}: unsupported statement {ln!r}")
        self.modvars[m.name] = ctx.local
        store = {}
        for nm, info in ctx.local.items():
            if info.get("param"):
                continue
            if info["dims"]:
                store[nm] = Array(eval(self._bounds_src(ctx, info["dims"]), {"M": self.M}), info["kind"])
            else:
                store[nm] = {"real": 0.0, "int": 0, "logical": False, "char": ""}[info["kind"]]
        self.M[m.name] = store

    # units ------------------------------------------------------------------
    def compile(self, u: Unit):
        if u.name in self.compiled:
            return self.compiled[u.name]
        ctx = Context(self, u)
        uses = [ln.split()[1].rstrip(",") for ln in u.body if ln.startswith("use ") and "omp_lib" not in ln]
        u.uses = uses + [x for x in u.uses if x not in uses]
        body = []
        ctx.namelists = {}
        for ln in u.body:
            m = re.match(r"namelist\s*/\s*(\w+)\s*/\s*(.*)$", ln)
            if m:  # namelist /group/ a, b: the members a namelist read sets
                ctx.namelists.setdefault(m.group(1), []).extend(x.strip() for x in m.group(2).split(","))
                continue
            if ln.startswith(("use ", "implicit")):
                continue
            if self._decl(ctx, ln):
                continue
            body.append(ln)
        args = u.args
        saves = {}  # local arrays and scalars persist across calls (-fno-automatic)
        py = [f"def _unit({', '.join('A_' + a for a in args)}):"]
        for a in args:
            info = ctx.local.get(a)
            if info is None:
                raise NameError(f"{u.name}: argument {a} undeclared")
            py.append(f"    L_{a} = A_{a}")
        for nm, info in ctx.local.items():
            if info.get("param") or nm in args:
                continue
            saves[nm] = info
            py.append(f"    L_{nm} = S[{nm!r}]")
        ind = 1
        for ln in body:
            for out, dind in self._stmt(ctx, ln):
                if dind < 0:
                    ind += dind
                py.append("    " * ind + out)
                if dind > 0:
                    ind += dind
        py.append("    " * 1 + "return _ret()")
        src_ret = ["def _ret():"]
        scal = [a for a in args if not ctx.local[a]["dims"]]
        src_ret.append("    return {" + ", ".join(f"{a!r}: L_{a}" for a in scal) + "}")
        # _ret needs the locals of _unit: emit it as a nested closure
        full = [py[0]] + ["    " + x for x in src_ret] + py[1:]
        full = self._fix_closure(full, args, saves)
        code = "\n".join(full)
        S = {}
        for nm, info in saves.items():
            if info["dims"]:
                S[nm] = Array(eval(self._bounds_src(ctx, info["dims"]), {"M": self.M}), info["kind"])
            else:
                S[nm] = {"real": 0.0, "int": 0, "logical": False, "char": ""}[info["kind"]]
        env = {"M": self.M, "S": S, "math": math, "_max": _max, "_min": _min, "_sq": _sq, "_pow": _pow,
               "_idiv": _idiv, "_mod": _mod, "_trim": _trim, "_range": _range, "P": self}
        try:
            exec(compile(code, f"<fortran {u.name}>", "exec"), env)
        except SyntaxError as e:
            raise SyntaxError(f"{u.name}: {e}\n{code}") from e
        fn = env["_unit"]
        self.compiled[u.name] = (fn, ctx, S)
        return self.compiled[u.name]

    @staticmethod
    def _fix_closure(lines, args, saves):
        # scalars assigned in the body are Python locals; _ret reads them as a
        # closure, and scalar saves are written back to S before returning
        out = []
        for ln in lines:
            if ln.strip() == "return _ret()":
                ind = ln[: len(ln) - len(ln.lstrip())]
                for nm, info in saves.items():
                    if not info["dims"]:
                        out.append(f"{ind}S[{nm!r}] = L_{nm}")
                out.append(ln)
            else:
                out.append(ln)
        return out

    def _assign_cast(self, kind, src, skind):
        if kind == "real" and skind != "real":
            return f"float({src})"
        if kind == "int" and skind == "real":
            return f"int({src})"
        return src

    def _stmt(self, ctx, ln):
        """Yield (python_line, indent_change)."""
        m = re.match(r"write\s*\(", ln)
        if m:
            return self._write(ctx, ln)
        if ln.startswith(("print", "close", "flush")):
            return [("pass", 0)]
        m = re.match(r"do\s+(\w+)\s*=\s*(.*)$", ln)
        if m:
            v = m.group(1)
            parts = Program._split_top(m.group(2))
            a, b = ctx.expr(parts[0])[0], ctx.expr(parts[1])[0]
            st = ctx.expr(parts[2])[0] if len(parts) > 2 else "1"
            vs, _ = ctx.var(v)
            return [(f"for {vs} in _range({a}, {b}, {st}):", 1)]
        if ln in ("end do", "enddo"):
            return [("pass", 0), ("#", -1)]
        m = re.match(r"if\s*\((.*)\)\s*then$", ln)
        if m:
            return [(f"if {ctx.expr(m.group(1))[0]}:", 1)]
        m = re.match(r"else\s*if\s*\((.*)\)\s*then$", ln)
        if m:
            return [("pass", 0), (f"elif {ctx.expr(m.group(1))[0]}:", -1), ("", 1)]
        if ln == "else":
            return [("pass", 0), ("else:", -1), ("", 1)]
        if ln in ("end if", "endif"):
            return [("pass", 0), ("#", -1)]
        m = re.match(r"if\s*\((.*)\)\s*(\w.*)$", ln)
        if m and self._balanced_if(ln):
            cond, rest = self._balanced_if(ln)
            inner = self._stmt(ctx, rest)
            out = [(f"if {ctx.expr(cond)[0]}:", 1)] + inner + [("#", -1)]
            return out
        if ln == "return":
            return [("return _ret()", 0)]
        if ln == "exit":
            return [("break", 0)]
        if ln == "cycle":
            return [("continue", 0)]
        if ln.startswith("stop"):
            return [("raise SystemExit(0)", 0)]
        m = re.match(r"call\s+(\w+)\s*(\((.*)\))?$", ln)
        if m:
            return self._call(ctx, m.group(1), m.group(3) or "")
        m = re.match(r"open\s*\((.*)\)$", ln)
        if m:
            parts = Program._split_top(m.group(1))
            unit = ctx.expr(parts[0])[0]
            fname = [p for p in parts if p.replace(" ", "").startswith("file=")][0].split("=", 1)[1]
            return [(f"P._open({unit}, {ctx.expr(fname)[0]})", 0)]
        m = re.match(r"read\s*\(\s*(\w+)\s*,\s*nml\s*=\s*(\w+)\s*\)$", ln)
        if m:  # a namelist read: the members the caller supplied (P.nml_values)
            group = m.group(2)
            out = [(f"_nl = P.nml({group!r})", 0)]
            for member in ctx.namelists.get(group, []):
                vs, _ = ctx.var(member)
                out.append((f"{vs} = _nl.get({member!r}, {vs})", 0))
            return out
        m = re.match(r"read\s*\((\w+)\s*,\s*\*\s*\)\s*(.*)$", ln)
        if m:
            unit = m.group(1)
            names = Program._split_top(m.group(2))
            targets = [self._lhs(ctx, n) for n in names]
            kinds = [k for _, k in targets]
            out = [(f"_vals = P._read({unit}, {kinds!r})", 0)]
            for q, (t, k) in enumerate(targets):
                out.append((f"{t} = _vals[{q}]", 0))
            return out
        m = re.match(r"(.+?)\s*=\s*(.+)$", ln)
        if m and not re.match(r"(if|do)\b", ln):
            lhs, lk = self._lhs(ctx, m.group(1))
            src, sk = ctx.expr(m.group(2))
            return [(f"{lhs} = {self._assign_cast(lk, src, sk)}", 0)]
        raise SyntaxError(f"{ctx.unit.name}: unsupported statement {ln!r}")

    @staticmethod
    def _balanced_if(ln):
        m = re.match(r"if\s*\(", ln)
        if not m:
            return None
        depth, i = 0, m.end() - 1
        for k in range(i, len(ln)):
            if ln[k] == "(":
                depth += 1
            elif ln[k] == ")":
                depth -= 1
                if depth == 0:
                    rest = ln[k + 1:].strip()
                    if not rest or rest == "then":
                        return None
                    return ln[i + 1:k], rest
        return None

    def _write(self, ctx, ln):
        """write(unit, fmt) items: the values are recorded (P.writes[unit],
        one list per record) instead of formatted; implied-do items
        (expr, v = a, b) expand in order."""
        depth, k0 = 0, ln.index("(")
        for k in range(k0, len(ln)):
            if ln[k] == "(":
                depth += 1
            elif ln[k] == ")":
                depth -= 1
                if depth == 0:
                    break
        spec = Program._split_top(ln[k0 + 1:k])
        unit = spec[0].strip()
        unit_src = repr("*") if unit == "*" else ctx.expr(unit)[0]
        items = Program._split_top(ln[k + 1:]) if ln[k + 1:].strip() else []
        parts = []
        for it in items:
            parts.append(self._write_item(ctx, it.strip()))
        return [(f"P.record({unit_src}, [{', '.join(parts)}])", 0)]

    def _write_item(self, ctx, it):
        m = re.match(r"\((.*)\)$", it)
        if m:
            inner = Program._split_top(m.group(1))
            # (items..., v = a, b[, s])
            for q in range(len(inner)):
                mm = re.match(r"(\w+)\s*=\s*(.*)$", inner[q])
                if mm:
                    v = mm.group(1)
                    lo = ctx.expr(mm.group(2))[0]
                    rest = inner[q + 1:]
                    hi = ctx.expr(rest[0])[0]
                    st = ctx.expr(rest[1])[0] if len(rest) > 1 else "1"
                    vs, _ = ctx.var(v)
                    body = ", ".join(self._write_item(ctx, x.strip()) for x in inner[:q])
                    return f"*[_x for {vs} in _range({lo}, {hi}, {st}) for _x in ({body},)]"
        return ctx.expr(it)[0]

    def _lhs(self, ctx, s):
        s = s.strip()
        m = re.match(r"(\w+)\s*\((.*)\)$", s)
        if m:
            info, _ = ctx.lookup(m.group(1))
            src, k = Expr(tokenize(s), ctx).parse()
            return src, k
        return ctx.var(s)

    def _call(self, ctx, name, argsrc):
        args = Program._split_top(argsrc) if argsrc.strip() else []
        srcs = []
        backs = []
        for q, a in enumerate(args):
            src, k = ctx.expr(a)
            srcs.append(src)
            if re.fullmatch(r"\w+", a.strip()):
                info, _ = ctx.lookup(a.strip())
                if info is not None and not info.get("param") and not info.get("dims"):
                    backs.append((q, src))
        call = f"_r = P.call({name!r}, [{', '.join(srcs)}])"
        out = [(call, 0)]
        for q, src in backs:
            out.append((f"{src} = _r[{q}] if _r is not None and _r[{q}] is not None else {src}", 0))
        return out

    # runtime ------------------------------------------------------------------
    def call(self, name, argvals):
        if name in self.stubs:
            res = self.stubs[name](self, *argvals)
            return res
        u = self.subs.get(name)
        if u is None:
            raise NameError(f"no subroutine {name}")
        fn, ctx, _ = self.compile(u)
        ret = fn(*argvals)
        return [ret.get(a) for a in u.args]

    def _open(self, unit, fname):
        name = fname.strip()
        if name in self.vfs:
            self.files[int(unit)] = self.vfs[name].splitlines()
        else:  # a file the program writes
            self.writes.setdefault(int(unit), [])

    def nml(self, group):
        """Values of namelist group `group` for a `read(u, nml=group)`."""
        return getattr(self, "nml_values", {}).get(group, {})

    def record(self, unit, values):
        if isinstance(unit, str) and unit != "*":
            # an internal write into a character variable (a file name's
            # step number): recorded, the variable itself is left unchanged
            self.writes.setdefault("internal", []).append(list(values))
            return
        self.writes.setdefault(unit if unit == "*" else int(unit), []).append(list(values))

    def _read(self, unit, kinds):
        lines = self.files[int(unit)]
        ln = lines.pop(0)
        toks = [t for t in re.split(r"[,\s]+", ln.strip()) if t]
        out = []
        for k, t in zip(kinds, toks):
            out.append(int(t) if k == "int" else float(t.replace("d", "e").replace("D", "e")))
        return out

    def run_main(self):
        u = self.main
        u.args = []
        fn, ctx, S = self.compile(u)
        fn()
        return S


def _range(a, b, s):
    return range(a, b + 1, s) if s > 0 else range(a, b - 1, s)
