"""A Lua 5.1 subset interpreter for D+'s scripted symmetries.

The reference runs a scripted symmetry's ``Populate(p, nlayers)`` in an
embedded Lua state with ``os`` and ``io`` removed (Backend/Backend/
Symmetry.cpp:404-521): ``p`` is the node's parameter matrix as a table of
rows (``p[layer][parameter]``, 1-based), and the result is a table of rows
``{x, y, z, alpha, beta, gamma}`` (nm, degrees) that the symmetry then uses
exactly as a ManualSymmetry uses its rows.  This module evaluates such
scripts without a Lua runtime: the statements (assignment, ``local``,
``if``/``elseif``/``else``, numeric and generic ``for``, ``while``,
``repeat``, ``function``, ``return``, ``break``, ``do``), expressions with
Lua's precedence, tables, closures and multiple results, and the library
functions scripts of this kind call (``math``, ``table``, ``string``
subsets, ``pairs``, ``ipairs``, ``error``, ``type``, ``tonumber``,
``tostring``, ``unpack``, ``assert``, ``print``).  There is no ``os``, ``io``,
``load`` or ``require``; a step budget ends runaway scripts with an error.

``populate(script, params)`` returns the rows as an (N, 6) array.
"""
from __future__ import annotations

import math
import re

import numpy as np


class LuaError(Exception):
    """A Lua runtime or syntax error (``error()`` in the script included)."""


# ---------------------------------------------------------------- values ----
class Table:
    __slots__ = ("h",)

    def __init__(self, h=None):
        self.h = h or {}

    def get(self, k):
        if isinstance(k, float) and k.is_integer():
            k = int(k)
        return self.h.get(k)

    def set(self, k, v):
        if k is None:
            raise LuaError("table index is nil")
        if isinstance(k, float):
            if k != k:
                raise LuaError("table index is NaN")
            if k.is_integer():
                k = int(k)
        if v is None:
            self.h.pop(k, None)
        else:
            self.h[k] = v

    def length(self):  # a border of the array part (Lua's #)
        n = 0
        while (n + 1) in self.h:
            n += 1
        return n


class Function:
    __slots__ = ("params", "vararg", "body", "scope", "name")

    def __init__(self, params, vararg, body, scope, name="?"):
        self.params, self.vararg, self.body, self.scope, self.name = params, vararg, body, scope, name


class _Return(Exception):
    def __init__(self, values):
        self.values = values


class _Break(Exception):
    pass


def _type(v):
    if v is None:
        return "nil"
    if isinstance(v, bool):
        return "boolean"
    if isinstance(v, (int, float)):
        return "number"
    if isinstance(v, str):
        return "string"
    if isinstance(v, Table):
        return "table"
    return "function"


def _truthy(v):
    return v is not None and v is not False


def _num_str(x):
    if isinstance(x, int) or (isinstance(x, float) and x.is_integer() and abs(x) < 1e15):
        return str(int(x))
    return "%.14g" % x


def _tostr(v):
    if v is None:
        return "nil"
    if v is True:
        return "true"
    if v is False:
        return "false"
    if isinstance(v, (int, float)):
        return _num_str(v)
    if isinstance(v, str):
        return v
    return "%s: 0x%08x" % (_type(v), id(v) & 0xffffffff)


def _tonum(v):
    if isinstance(v, bool):
        return None
    if isinstance(v, (int, float)):
        return v
    if isinstance(v, str):
        s = v.strip()
        try:
            return int(s, 16) if s.lower().startswith(("0x", "-0x")) else float(s)
        except ValueError:
            return None
    return None


def _arith_operand(v, op):
    n = _tonum(v) if isinstance(v, str) else (v if isinstance(v, (int, float)) and not isinstance(v, bool) else None)
    if n is None:
        raise LuaError(f"attempt to perform arithmetic ({op}) on a {_type(v)} value")
    return n


# ----------------------------------------------------------------- lexer ----
_TOKEN = re.compile(r"""
    (?P<ws>\s+)
  | (?P<comment>--(?:\[(?P<eq>=*)\[[\s\S]*?\](?P=eq)\]|[^\n]*))
  | (?P<long>\[(?P<leq>=*)\[[\s\S]*?\](?P=leq)\])
  | (?P<num>0[xX][0-9a-fA-F]+|(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?)
  | (?P<name>[A-Za-z_][A-Za-z_0-9]*)
  | (?P<str>"(?:\\.|[^"\\\n])*"|'(?:\\.|[^'\\\n])*')
  | (?P<op>\.\.\.|\.\.|==|~=|<=|>=|[-+*/%^\#<>=(){}\[\];:,.])
""", re.X)

_KEYWORDS = {"and", "break", "do", "else", "elseif", "end", "false", "for", "function", "if", "in", "local", "nil",
             "not", "or", "repeat", "return", "then", "true", "until", "while"}

_ESC = {"n": "\n", "t": "\t", "r": "\r", "a": "\a", "b": "\b", "f": "\f", "v": "\v", "\\": "\\", '"': '"', "'": "'",
        "\n": "\n"}


def _unescape(s):
    out, i = [], 0
    while i < len(s):
        c = s[i]
        if c == "\\" and i + 1 < len(s):
            d = s[i + 1]
            if d.isdigit():
                j = i + 1
                while j < len(s) and j < i + 4 and s[j].isdigit():
                    j += 1
                out.append(chr(int(s[i + 1:j])))
                i = j
                continue
            out.append(_ESC.get(d, d))
            i += 2
        else:
            out.append(c)
            i += 1
    return "".join(out)


def _tokens(src):
    toks, pos, line = [], 0, 1
    while pos < len(src):
        m = _TOKEN.match(src, pos)
        if not m:
            raise LuaError(f"line {line}: unexpected symbol near {src[pos:pos + 10]!r}")
        kind = m.lastgroup
        text = m.group(0)
        if kind == "num":
            toks.append(("num", float(int(text, 16)) if text.lower().startswith("0x") else float(text), line))
        elif kind == "name":
            toks.append(("kw" if text in _KEYWORDS else "name", text, line))
        elif kind == "str":
            toks.append(("str", _unescape(text[1:-1]), line))
        elif kind == "long":
            body = text[len(m.group("leq")) + 2:-(len(m.group("leq")) + 2)]
            toks.append(("str", body[1:] if body.startswith("\n") else body, line))
        elif kind == "op":
            toks.append(("op", text, line))
        line += text.count("\n")
        pos = m.end()
    toks.append(("eof", None, line))
    return toks


# ---------------------------------------------------------------- parser ----
# Nodes are tuples ("kind", ...).
_BINPRI = {"or": (1, 1), "and": (2, 2), "<": (3, 3), ">": (3, 3), "<=": (3, 3), ">=": (3, 3), "~=": (3, 3),
           "==": (3, 3), "..": (5, 4), "+": (6, 6), "-": (6, 6), "*": (7, 7), "/": (7, 7), "%": (7, 7),
           "^": (10, 9)}
_UNARY_PRI = 8


class _Parser:
    def __init__(self, src):
        self.t = _tokens(src)
        self.i = 0

    def peek(self, k=0):
        return self.t[self.i + k]

    def check(self, kind, val=None):
        tk = self.t[self.i]
        return tk[0] == kind and (val is None or tk[1] == val)

    def accept(self, kind, val=None):
        if self.check(kind, val):
            self.i += 1
            return True
        return False

    def expect(self, kind, val=None):
        tk = self.t[self.i]
        if tk[0] != kind or (val is not None and tk[1] != val):
            raise LuaError(f"line {tk[2]}: '{val or kind}' expected near {tk[1]!r}")
        self.i += 1
        return tk[1]

    def block_end(self):
        tk = self.t[self.i]
        return tk[0] == "eof" or (tk[0] == "kw" and tk[1] in ("end", "else", "elseif", "until"))

    def block(self):
        stats = []
        while not self.block_end():
            if self.check("kw", "return"):
                self.i += 1
                vals = [] if (self.block_end() or self.check("op", ";")) else self.explist()
                self.accept("op", ";")
                stats.append(("return", vals))
                break
            if self.accept("kw", "break"):
                stats.append(("break",))
                self.accept("op", ";")
                break
            st = self.statement()
            if st is not None:
                stats.append(st)
            self.accept("op", ";")
        return stats

    def statement(self):
        if self.accept("kw", "if"):
            arms = []
            cond = self.expr()
            self.expect("kw", "then")
            arms.append((cond, self.block()))
            other = None
            while True:
                if self.accept("kw", "elseif"):
                    cond = self.expr()
                    self.expect("kw", "then")
                    arms.append((cond, self.block()))
                elif self.accept("kw", "else"):
                    other = self.block()
                    self.expect("kw", "end")
                    break
                else:
                    self.expect("kw", "end")
                    break
            return ("if", arms, other)
        if self.accept("kw", "while"):
            cond = self.expr()
            self.expect("kw", "do")
            body = self.block()
            self.expect("kw", "end")
            return ("while", cond, body)
        if self.accept("kw", "do"):
            body = self.block()
            self.expect("kw", "end")
            return ("do", body)
        if self.accept("kw", "repeat"):
            body = self.block()
            self.expect("kw", "until")
            return ("repeat", body, self.expr())
        if self.accept("kw", "for"):
            name = self.expect("name")
            if self.accept("op", "="):
                a = self.expr()
                self.expect("op", ",")
                b = self.expr()
                c = self.expr() if self.accept("op", ",") else None
                self.expect("kw", "do")
                body = self.block()
                self.expect("kw", "end")
                return ("fornum", name, a, b, c, body)
            names = [name]
            while self.accept("op", ","):
                names.append(self.expect("name"))
            self.expect("kw", "in")
            exps = self.explist()
            self.expect("kw", "do")
            body = self.block()
            self.expect("kw", "end")
            return ("forin", names, exps, body)
        if self.accept("kw", "function"):
            target = ("name", self.expect("name"))
            fname = target[1]
            method = False
            while self.check("op", ".") or self.check("op", ":"):
                sep = self.peek()[1]
                self.i += 1
                key = self.expect("name")
                fname += sep + key
                target = ("index", target, ("const", key))
                if sep == ":":
                    method = True
                    break
            f = self.funcbody(fname, method)
            return ("assign", [target], [f])
        if self.accept("kw", "local"):
            if self.accept("kw", "function"):
                name = self.expect("name")
                return ("localfunc", name, self.funcbody(name, False))
            names = [self.expect("name")]
            while self.accept("op", ","):
                names.append(self.expect("name"))
            exps = self.explist() if self.accept("op", "=") else []
            return ("local", names, exps)
        # assignment or call
        e = self.suffixed()
        if self.check("op", "=") or self.check("op", ","):
            targets = [e]
            while self.accept("op", ","):
                targets.append(self.suffixed())
            self.expect("op", "=")
            for tg in targets:
                if tg[0] not in ("name", "index"):
                    raise LuaError(f"line {self.peek()[2]}: cannot assign to this expression")
            return ("assign", targets, self.explist())
        if e[0] not in ("call", "method"):
            raise LuaError(f"line {self.peek()[2]}: syntax error near {self.peek()[1]!r}")
        return ("exprstat", e)

    def funcbody(self, name, method):
        self.expect("op", "(")
        params, vararg = (["self"] if method else []), False
        if not self.check("op", ")"):
            while True:
                if self.accept("op", "..."):
                    vararg = True
                    break
                params.append(self.expect("name"))
                if not self.accept("op", ","):
                    break
        self.expect("op", ")")
        body = self.block()
        self.expect("kw", "end")
        return ("function", params, vararg, body, name)

    def explist(self):
        out = [self.expr()]
        while self.accept("op", ","):
            out.append(self.expr())
        return out

    def primary(self):
        if self.accept("op", "("):
            e = self.expr()
            self.expect("op", ")")
            return ("paren", e)
        return ("name", self.expect("name"))

    def suffixed(self):
        e = self.primary()
        while True:
            if self.accept("op", "."):
                e = ("index", e, ("const", self.expect("name")))
            elif self.accept("op", "["):
                k = self.expr()
                self.expect("op", "]")
                e = ("index", e, k)
            elif self.accept("op", ":"):
                name = self.expect("name")
                e = ("method", e, name, self.args())
            elif self.check("op", "(") or self.check("op", "{") or self.check("str"):
                e = ("call", e, self.args())
            else:
                return e

    def args(self):
        if self.check("str"):
            return [("const", self.expect("str"))]
        if self.check("op", "{"):
            return [self.table()]
        self.expect("op", "(")
        if self.accept("op", ")"):
            return []
        a = self.explist()
        self.expect("op", ")")
        return a

    def table(self):
        self.expect("op", "{")
        items = []  # ("pos", e) | ("key", k, e)
        while not self.check("op", "}"):
            if self.check("op", "["):
                self.i += 1
                k = self.expr()
                self.expect("op", "]")
                self.expect("op", "=")
                items.append(("key", k, self.expr()))
            elif self.check("name") and self.peek(1)[0] == "op" and self.peek(1)[1] == "=":
                k = self.expect("name")
                self.expect("op", "=")
                items.append(("key", ("const", k), self.expr()))
            else:
                items.append(("pos", self.expr()))
            if not (self.accept("op", ",") or self.accept("op", ";")):
                break
        self.expect("op", "}")
        return ("table", items)

    def simple(self):
        tk = self.peek()
        if tk[0] == "num":
            self.i += 1
            return ("const", tk[1])
        if tk[0] == "str":
            self.i += 1
            return ("const", tk[1])
        if tk[0] == "kw" and tk[1] in ("nil", "true", "false"):
            self.i += 1
            return ("const", {"nil": None, "true": True, "false": False}[tk[1]])
        if tk[0] == "op" and tk[1] == "...":
            self.i += 1
            return ("vararg",)
        if tk[0] == "op" and tk[1] == "{":
            return self.table()
        if tk[0] == "kw" and tk[1] == "function":
            self.i += 1
            return self.funcbody("anonymous", False)
        return self.suffixed()

    def expr(self, limit=0):
        tk = self.peek()
        if (tk[0] == "kw" and tk[1] == "not") or (tk[0] == "op" and tk[1] in ("-", "#")):
            self.i += 1
            left = ("unop", tk[1], self.expr(_UNARY_PRI))
        else:
            left = self.simple()
        while True:
            tk = self.peek()
            op = tk[1] if tk[0] in ("op", "kw") else None
            if op not in _BINPRI or _BINPRI[op][0] <= limit:
                return left
            self.i += 1
            right = self.expr(_BINPRI[op][1])
            left = ("binop", op, left, right)


# ----------------------------------------------------------- interpreter ----
class _Scope:
    __slots__ = ("vars", "parent", "varargs")

    def __init__(self, parent=None, varargs=None):
        self.vars, self.parent = {}, parent
        self.varargs = varargs if varargs is not None else (parent.varargs if parent else [])

    def find(self, name):
        s = self
        while s is not None:
            if name in s.vars:
                return s
            s = s.parent
        return None


class Interpreter:
    """One Lua state: globals with the library subset; ``run`` executes a chunk."""

    def __init__(self, max_steps: int = 50_000_000):
        self.steps, self.max_steps = 0, max_steps
        self.G = Table()
        g = self.G.set
        g("print", lambda *a: [])
        g("error", self._error)
        g("assert", self._assert)
        g("type", lambda v=None, *a: [_type(v)])
        g("tostring", lambda v=None, *a: [_tostr(v)])
        g("tonumber", self._tonumber)
        g("pairs", self._pairs)
        g("ipairs", self._ipairs)
        g("next", self._next)
        g("unpack", self._unpack)
        g("select", self._select)
        g("rawget", lambda t, k, *a: [t.get(k)])
        g("rawset", lambda t, k, v, *a: (t.set(k, v), [t])[1])
        m = Table()
        for name, f in {"abs": abs, "acos": math.acos, "asin": math.asin, "atan": math.atan, "atan2": math.atan2,
                        "ceil": math.ceil, "cos": math.cos, "cosh": math.cosh, "deg": math.degrees, "exp": math.exp,
                        "floor": math.floor, "log10": math.log10, "rad": math.radians, "sin": math.sin,
                        "sinh": math.sinh, "sqrt": math.sqrt, "tan": math.tan, "tanh": math.tanh}.items():
            m.set(name, self._math1(f))
        m.set("log", lambda x, *a: [math.log(_arith_operand(x, "log"))])
        m.set("pow", lambda x, y, *a: [math.pow(_arith_operand(x, "pow"), _arith_operand(y, "pow"))])
        m.set("fmod", lambda x, y, *a: [math.fmod(_arith_operand(x, "fmod"), _arith_operand(y, "fmod"))])
        m.set("modf", lambda x, *a: [float(math.trunc(x)), x - math.trunc(x)])
        m.set("max", lambda *a: [max(_arith_operand(x, "max") for x in a)])
        m.set("min", lambda *a: [min(_arith_operand(x, "min") for x in a)])
        m.set("pi", math.pi)
        m.set("huge", math.inf)
        g("math", m)
        t = Table()
        t.set("getn", lambda tb, *a: [float(tb.length())])
        t.set("insert", self._tinsert)
        t.set("remove", self._tremove)
        t.set("concat", self._tconcat)
        g("table", t)
        s = Table()
        s.set("format", self._format)
        s.set("len", lambda x, *a: [float(len(x))])
        s.set("sub", self._ssub)
        s.set("rep", lambda x, n, *a: [x * int(n)])
        s.set("upper", lambda x, *a: [x.upper()])
        s.set("lower", lambda x, *a: [x.lower()])
        g("string", s)

    # -- library --
    @staticmethod
    def _math1(f):
        return lambda x=None, *a: [float(f(_arith_operand(x, "math")))]

    @staticmethod
    def _error(msg=None, *a):
        raise LuaError(_tostr(msg))

    @staticmethod
    def _assert(v=None, msg="assertion failed!", *a):
        if not _truthy(v):
            raise LuaError(_tostr(msg))
        return [v, msg, *a]

    @staticmethod
    def _tonumber(v=None, base=None, *a):
        if base is not None and isinstance(v, str):
            try:
                return [float(int(v.strip(), int(base)))]
            except ValueError:
                return [None]
        n = _tonum(v)
        return [float(n) if n is not None else None]

    @staticmethod
    def _next(t, k=None, *a):
        keys = list(t.h.keys())
        if k is None:
            i = 0
        else:
            if isinstance(k, float) and k.is_integer():
                k = int(k)
            i = keys.index(k) + 1
        if i >= len(keys):
            return [None]
        kk = keys[i]
        return [float(kk) if isinstance(kk, int) else kk, t.h[kk]]

    def _pairs(self, t, *a):
        return [self.G.get("next"), t, None]

    @staticmethod
    def _ipairs(t, *a):
        def it(tb, i, *rest):
            v = tb.get(i + 1)
            return [None] if v is None else [i + 1.0, v]
        return [it, t, 0.0]

    @staticmethod
    def _unpack(t, i=1, j=None, *a):
        j = t.length() if j is None else int(j)
        return [t.get(k) for k in range(int(i), j + 1)]

    @staticmethod
    def _select(n, *a):
        if n == "#":
            return [float(len(a))]
        return list(a[int(n) - 1:])

    @staticmethod
    def _tinsert(t, *a):
        if len(a) == 1:
            t.set(t.length() + 1, a[0])
        else:
            pos, v = int(a[0]), a[1]
            for k in range(t.length(), pos - 1, -1):
                t.set(k + 1, t.get(k))
            t.set(pos, v)
        return []

    @staticmethod
    def _tremove(t, pos=None, *a):
        n = t.length()
        if n == 0:
            return [None]
        pos = n if pos is None else int(pos)
        v = t.get(pos)
        for k in range(pos, n):
            t.set(k, t.get(k + 1))
        t.set(n, None)
        return [v]

    @staticmethod
    def _tconcat(t, sep="", i=1, j=None, *a):
        j = t.length() if j is None else int(j)
        return [sep.join(_tostr(t.get(k)) for k in range(int(i), j + 1))]

    @staticmethod
    def _ssub(s, i=1, j=-1, *a):
        n = len(s)
        i, j = int(i), int(j)
        if i < 0:
            i = max(n + i + 1, 1)
        elif i == 0:
            i = 1
        if j < 0:
            j = n + j + 1
        elif j > n:
            j = n
        return [s[i - 1:j] if i <= j else ""]

    @staticmethod
    def _format(fmt, *args):
        ai = 0

        def rep(m):
            nonlocal ai
            spec = m.group(0)
            if spec == "%%":
                return "%"
            v = args[ai]
            ai += 1
            conv = spec[-1]
            if conv in "dioxXuc":
                v = int(v)
                spec = spec[:-1] + ("d" if conv in "iu" else conv)
            elif conv == "s":
                v = _tostr(v)
            elif conv == "q":
                return '"' + _tostr(v).replace("\\", "\\\\").replace('"', '\\"') + '"'
            return spec % v
        return [re.sub(r"%(?:%|[-+ #0]*\d*(?:\.\d+)?[diouxXeEfgGqsc])", rep, fmt)]

    # -- evaluation --
    def tick(self):
        self.steps += 1
        if self.steps > self.max_steps:
            raise LuaError("script exceeded its step budget")

    def run(self, src: str):
        chunk = _Parser(src).block()
        try:
            self.exec_block(chunk, _Scope())
        except _Return:
            pass
        except RecursionError:
            raise LuaError("stack overflow") from None

    def call(self, f, args):
        self.tick()
        if isinstance(f, Function):
            scope = _Scope(f.scope, varargs=list(args[len(f.params):]) if f.vararg else [])
            for i, p in enumerate(f.params):
                scope.vars[p] = args[i] if i < len(args) else None
            try:
                self.exec_block(f.body, scope)
            except _Return as r:
                return r.values
            return []
        if callable(f):
            r = f(*args)
            return list(r) if r is not None else []
        raise LuaError(f"attempt to call a {_type(f)} value")

    def exec_block(self, stats, scope):
        for st in stats:
            self.exec(st, scope)

    def assign(self, target, value, scope):
        if target[0] == "name":
            s = scope.find(target[1])
            if s is not None:
                s.vars[target[1]] = value
            else:
                self.G.set(target[1], value)
        else:
            t = self.eval(target[1], scope)
            if not isinstance(t, Table):
                raise LuaError(f"attempt to index a {_type(t)} value")
            t.set(self.eval(target[2], scope), value)

    def exec(self, st, scope):
        self.tick()
        k = st[0]
        if k == "assign":
            vals = self.eval_list(st[2], scope)
            for i, tg in enumerate(st[1]):
                self.assign(tg, vals[i] if i < len(vals) else None, scope)
        elif k == "local":
            vals = self.eval_list(st[2], scope)
            for i, name in enumerate(st[1]):
                scope.vars[name] = vals[i] if i < len(vals) else None
        elif k == "localfunc":
            scope.vars[st[1]] = None
            scope.vars[st[1]] = self.eval(st[2], scope)
        elif k == "exprstat":
            self.eval_multi(st[1], scope)
        elif k == "if":
            for cond, body in st[1]:
                if _truthy(self.eval(cond, scope)):
                    self.exec_block(body, _Scope(scope))
                    return
            if st[2] is not None:
                self.exec_block(st[2], _Scope(scope))
        elif k == "while":
            try:
                while _truthy(self.eval(st[1], scope)):
                    self.tick()
                    self.exec_block(st[2], _Scope(scope))
            except _Break:
                pass
        elif k == "repeat":
            try:
                while True:
                    self.tick()
                    inner = _Scope(scope)
                    self.exec_block(st[1], inner)
                    if _truthy(self.eval(st[2], inner)):
                        break
            except _Break:
                pass
        elif k == "do":
            self.exec_block(st[1], _Scope(scope))
        elif k == "fornum":
            a = _arith_operand(self.eval(st[2], scope), "for")
            b = _arith_operand(self.eval(st[3], scope), "for")
            c = 1.0 if st[4] is None else _arith_operand(self.eval(st[4], scope), "for")
            if c == 0:
                raise LuaError("'for' step is zero")
            v = float(a)
            try:
                while (c > 0 and v <= b) or (c < 0 and v >= b):
                    self.tick()
                    inner = _Scope(scope)
                    inner.vars[st[1]] = v
                    self.exec_block(st[5], inner)
                    v += c
            except _Break:
                pass
        elif k == "forin":
            vals = self.eval_list(st[2], scope)
            f, s, ctl = (vals + [None, None, None])[:3]
            try:
                while True:
                    self.tick()
                    r = self.call(f, [s, ctl])
                    if not r or r[0] is None:
                        break
                    ctl = r[0]
                    inner = _Scope(scope)
                    for i, name in enumerate(st[1]):
                        inner.vars[name] = r[i] if i < len(r) else None
                    self.exec_block(st[3], inner)
            except _Break:
                pass
        elif k == "return":
            raise _Return(self.eval_list(st[1], scope))
        elif k == "break":
            raise _Break()
        else:
            raise LuaError(f"unknown statement {k}")

    def eval_list(self, exps, scope):
        out = []
        for i, e in enumerate(exps):
            if i == len(exps) - 1:
                out.extend(self.eval_multi(e, scope))
            else:
                out.append(self.eval(e, scope))
        return out

    def eval_multi(self, e, scope):
        k = e[0]
        if k == "call":
            f = self.eval(e[1], scope)
            return self.call(f, self.eval_list(e[2], scope))
        if k == "method":
            obj = self.eval(e[1], scope)
            if isinstance(obj, str):  # ("s"):upper() through the string table
                f = self.G.get("string").get(e[2])
            elif isinstance(obj, Table):
                f = obj.get(e[2])
            else:
                raise LuaError(f"attempt to index a {_type(obj)} value")
            return self.call(f, [obj] + self.eval_list(e[3], scope))
        if k == "vararg":
            return list(scope.varargs)
        return [self.eval(e, scope)]

    def eval(self, e, scope):
        k = e[0]
        if k == "const":
            return e[1]
        if k == "name":
            s = scope.find(e[1])
            return s.vars[e[1]] if s is not None else self.G.get(e[1])
        if k == "index":
            t = self.eval(e[1], scope)
            key = self.eval(e[2], scope)
            if isinstance(t, Table):
                return t.get(key)
            if isinstance(t, str):  # string methods through the string table
                return self.G.get("string").get(key)
            raise LuaError(f"attempt to index a {_type(t)} value")
        if k in ("call", "method", "vararg"):
            r = self.eval_multi(e, scope)
            return r[0] if r else None
        if k == "paren":
            return self.eval(e[1], scope)
        if k == "function":
            return Function(e[1], e[2], e[3], scope, e[4])
        if k == "table":
            t = Table()
            n = 1
            for idx, it in enumerate(e[1]):
                if it[0] == "key":
                    t.set(self.eval(it[1], scope), self.eval(it[2], scope))
                elif idx == len(e[1]) - 1:
                    for v in self.eval_multi(it[1], scope):
                        t.set(n, v)
                        n += 1
                else:
                    t.set(n, self.eval(it[1], scope))
                    n += 1
            return t
        if k == "unop":
            v = self.eval(e[2], scope)
            if e[1] == "not":
                return not _truthy(v)
            if e[1] == "-":
                return -_arith_operand(v, "unm")
            if isinstance(v, Table):
                return float(v.length())
            if isinstance(v, str):
                return float(len(v))
            raise LuaError(f"attempt to get length of a {_type(v)} value")
        if k == "binop":
            op = e[1]
            if op == "and":
                a = self.eval(e[2], scope)
                return self.eval(e[3], scope) if _truthy(a) else a
            if op == "or":
                a = self.eval(e[2], scope)
                return a if _truthy(a) else self.eval(e[3], scope)
            a, b = self.eval(e[2], scope), self.eval(e[3], scope)
            return self.binop(op, a, b)
        raise LuaError(f"unknown expression {k}")

    @staticmethod
    def binop(op, a, b):
        if op == "..":
            for v in (a, b):
                if not isinstance(v, (str, int, float)) or isinstance(v, bool):
                    raise LuaError(f"attempt to concatenate a {_type(v)} value")
            return (a if isinstance(a, str) else _num_str(a)) + (b if isinstance(b, str) else _num_str(b))
        if op == "==":
            return a == b and _type(a) == _type(b) if not (isinstance(a, Table) or isinstance(b, Table)) else a is b
        if op == "~=":
            return not Interpreter.binop("==", a, b)
        if op in ("<", "<=", ">", ">="):
            if isinstance(a, str) and isinstance(b, str):
                pass
            elif not (isinstance(a, (int, float)) and isinstance(b, (int, float))) or isinstance(a, bool) or \
                    isinstance(b, bool):
                raise LuaError(f"attempt to compare {_type(a)} with {_type(b)}")
            return {"<": a < b, "<=": a <= b, ">": a > b, ">=": a >= b}[op]
        x, y = _arith_operand(a, op), _arith_operand(b, op)
        if op == "+":
            return float(x + y)
        if op == "-":
            return float(x - y)
        if op == "*":
            return float(x * y)
        if op == "/":
            if y == 0:
                if x == 0 or x != x:
                    return math.nan
                return math.copysign(math.inf, x) * math.copysign(1.0, y)
            return float(x / y)
        if op == "%":
            if y == 0:
                return math.nan
            return float(x - math.floor(x / y) * y)
        if op == "^":
            return float(math.pow(x, y))
        raise LuaError(f"unknown operator {op}")


def to_table(rows) -> Table:
    """A Lua table of tables from a 2-D list (1-based rows and columns)."""
    t = Table()
    for i, row in enumerate(rows):
        r = Table()
        for j, v in enumerate(row):
            r.set(j + 1, float(v))
        t.set(i + 1, r)
    return t


def populate(script: str, params, n_layers: int | None = None) -> np.ndarray:
    """Run the script, then ``Populate(p, nlayers)`` with ``p`` = params (a
    [layer][parameter] list) as the reference's LuaSymmetry::PreCalculate does
    (Backend/Backend/Symmetry.cpp:463-521); returns its rows as an (N, 6)
    array of x, y, z (nm), alpha, beta, gamma (degrees).  Missing or
    non-numeric entries of a row are 0 (getlocrot, Symmetry.cpp:441-461)."""
    L = Interpreter()
    L.run(script)
    if not isinstance(L.G.get("Information"), Table) or not isinstance(L.G.get("Populate"), Function):
        raise LuaError("a scripted symmetry needs an Information table and a Populate function")
    params = [list(r) for r in params]
    nl = len(params) if n_layers is None else int(n_layers)
    r = L.call(L.G.get("Populate"), [to_table(params), float(nl)])
    res = r[0] if r else None
    if not isinstance(res, Table):
        raise LuaError("Populate did not return a table")
    rows = np.zeros((res.length(), 6))
    for i in range(res.length()):
        row = res.get(i + 1)
        if not isinstance(row, Table):
            continue
        for j in range(6):
            v = row.get(j + 1)
            if isinstance(v, (int, float)) and not isinstance(v, bool):
                rows[i, j] = v
    return rows
