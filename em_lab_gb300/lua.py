"""A Lua 5.4 subset for the scene scripts: lexer, parser and a compiler to Python closures.

The reference runs its scene files (scenes/*.lua) in a sandboxed Lua 5.4 state with a vector
prelude (src/ScriptEngine.cpp:2194-2244) and the scene API (:2286-2314). Lua is not available here,
so this module implements the language the scenes and the prelude use: locals and closures with
upvalues, multiple assignment and returns, varargs, numeric and generic `for`, `while`, `repeat`,
`if`, method calls, table constructors, metatables (__index, __newindex, __add, __sub, __mul,
__div, __mod, __pow, __unm, __idiv, __concat, __len, __eq, __lt, __le, __call, __tostring), the
integer/float number subtypes of Lua 5.4, and the base, string, math and table libraries the
scenes call. `goto` is not supported. math.random follows Lua 5.4's xoshiro256** generator and
its seeding, so seeded scenes draw the same numbers as the reference.
"""
from __future__ import annotations

import math
import re
import struct

__all__ = ["LuaError", "LuaTable", "LuaFunction", "Interpreter", "tostr", "lua_type"]


class LuaError(Exception):
    """A Lua runtime or syntax error; `value` is the error object."""

    def __init__(self, value, traceback=None):
        super().__init__(value if isinstance(value, str) else tostr(value))
        self.value = value
        self.traceback = traceback


# ------------------------------------------------------------------------------------------ values
class LuaTable:
    __slots__ = ("hash", "meta")

    def __init__(self, items=None, meta=None):
        self.hash = {}
        self.meta = meta
        if items:
            for i, v in enumerate(items, 1):
                if v is not None:
                    self.hash[i] = v

    def rawget(self, k):
        return self.hash.get(_key(k))

    def rawset(self, k, v):
        k = _key(k)
        if v is None:
            self.hash.pop(k, None)
        else:
            self.hash[k] = v

    def length(self):
        h = self.hash
        if 1 not in h:
            return 0
        n = len(h)
        if n in h and (n + 1) not in h:  # pure sequence: the common case
            return n
        i = 1
        while (i + 1) in h:
            i += 1
        return i

    def array(self):
        return [self.hash[i] for i in range(1, self.length() + 1)]


class _BoolKey:
    """Table key for booleans (Python's True == 1 would collide with the integer key 1)."""
    __slots__ = ("v",)

    def __init__(self, v):
        self.v = v

    def __eq__(self, o):
        return isinstance(o, _BoolKey) and o.v == self.v

    def __hash__(self):
        return hash(("bool", self.v))


_TRUE, _FALSE = _BoolKey(True), _BoolKey(False)


def _key(k):
    if k is True:
        return _TRUE
    if k is False:
        return _FALSE
    if type(k) is float and k.is_integer():
        return int(k)
    if k is None:
        raise LuaError("table index is nil")
    if type(k) is float and k != k:
        raise LuaError("table index is NaN")
    return k


def _unkey(k):
    return k.v if isinstance(k, _BoolKey) else k


class LuaFunction:
    __slots__ = ("name", "call")

    def __init__(self, name, call):
        self.name = name
        self.call = call  # python callable: list of args -> list of results


def lua_type(v):
    if v is None:
        return "nil"
    t = type(v)
    if t is bool:
        return "boolean"
    if t is int or t is float:
        return "number"
    if t is str:
        return "string"
    if t is LuaTable:
        return "table"
    if t is LuaFunction or callable(v):
        return "function"
    return "userdata"


def _fmt_float(x: float) -> str:
    if x != x:
        return "nan" if math.copysign(1.0, x) > 0 else "-nan"
    if x in (math.inf, -math.inf):
        return "inf" if x > 0 else "-inf"
    s = "%.14g" % x
    if re.fullmatch(r"-?\d+", s):
        s += ".0"
    return s


def tostr(v, interp=None) -> str:
    if v is None:
        return "nil"
    if v is True:
        return "true"
    if v is False:
        return "false"
    t = type(v)
    if t is int:
        return str(v)
    if t is float:
        return _fmt_float(v)
    if t is str:
        return v
    if t is LuaTable:
        if interp is not None and v.meta is not None:
            h = v.meta.rawget("__tostring")
            if h is not None:
                r = interp.call(h, [v])
                return tostr(r[0] if r else None)
            name = v.meta.rawget("__name")
            if isinstance(name, str):
                return f"{name}: 0x{id(v):08x}"
        return f"table: 0x{id(v):08x}"
    if t is LuaFunction:
        return f"function: 0x{id(v):08x}"
    return f"userdata: 0x{id(v):08x}"


_NUM_RE = re.compile(r"\s*([-+]?)(0[xX][0-9a-fA-F]*\.?[0-9a-fA-F]*(?:[pP][-+]?\d+)?|(?:\d+\.?\d*|\.\d+)(?:[eE][-+]?\d+)?)\s*$")


def str2number(s: str):
    m = _NUM_RE.match(s)
    if not m:
        s2 = s.strip().lower()
        if s2 in ("inf", "-inf", "nan"):
            return None
        return None
    sign, body = m.group(1), m.group(2)
    neg = sign == "-"
    if body[:2] in ("0x", "0X"):
        if "." in body or "p" in body.lower():
            v = float.fromhex(body)
            return -v if neg else v
        v = int(body, 16) & 0xFFFFFFFFFFFFFFFF
        if v >= 1 << 63:
            v -= 1 << 64
        return -v if neg else v
    if re.fullmatch(r"\d+", body):
        v = int(body)
        if v < (1 << 63):
            return -v if neg else v
        return -float(body) if neg else float(body)
    v = float(body)
    return -v if neg else v


def tonum(v):
    t = type(v)
    if t is int or t is float:
        return v
    if t is str:
        return str2number(v)
    return None


def toint(v):
    """Integer value of v if it has an exact integer representation (Lua's lua_tointegerx)."""
    t = type(v)
    if t is int:
        return v
    if t is float:
        if v.is_integer():
            return int(v)
        return None
    if t is str:
        n = str2number(v)
        return toint(n) if n is not None else None
    return None


def _wrap64(v: int) -> int:
    v &= 0xFFFFFFFFFFFFFFFF
    return v - (1 << 64) if v >= 1 << 63 else v


# ------------------------------------------------------------------------------------------ lexer
_KEYWORDS = {"and", "break", "do", "else", "elseif", "end", "false", "for", "function", "goto", "if", "in",
             "local", "nil", "not", "or", "repeat", "return", "then", "true", "until", "while"}
_OPS = ["...", "..", "==", "~=", "<=", ">=", "//", "::", "<<", ">>", "+", "-", "*", "/", "%", "^", "#", "&", "~",
        "|", "<", ">", "=", "(", ")", "{", "}", "[", "]", ";", ":", ",", "."]
_ESC = {"n": "\n", "t": "\t", "r": "\r", "a": "\a", "b": "\b", "f": "\f", "v": "\v", "\\": "\\", '"': '"',
        "'": "'", "\n": "\n"}


class Tok:
    __slots__ = ("kind", "val", "line")

    def __init__(self, kind, val, line):
        self.kind, self.val, self.line = kind, val, line

    def __repr__(self):
        return f"{self.kind}:{self.val!r}@{self.line}"


def tokenize(src: str, chunk: str):
    toks = []
    i, n, line = 0, len(src), 1
    if src.startswith("#"):  # shebang line
        while i < n and src[i] != "\n":
            i += 1

    def err(msg):
        raise LuaError(f"{chunk}:{line}: {msg}")

    def long_bracket(j):
        """Level of a long bracket [==[ at j, or -1."""
        if src[j] != "[":
            return -1
        k = j + 1
        while k < n and src[k] == "=":
            k += 1
        return k - j - 1 if k < n and src[k] == "[" else -1

    def read_long(j, level):
        nonlocal line
        start = j + level + 2
        close = "]" + "=" * level + "]"
        end = src.find(close, start)
        if end < 0:
            err("unfinished long string/comment")
        body = src[start:end]
        line += body.count("\n")
        if body.startswith("\r\n"):
            body = body[2:]
        elif body.startswith("\n"):
            body = body[1:]
        return body, end + len(close)

    while i < n:
        c = src[i]
        if c == "\n":
            line += 1
            i += 1
            continue
        if c in " \t\r\f\v":
            i += 1
            continue
        if src.startswith("--", i):
            lv = long_bracket(i + 2) if i + 2 < n else -1
            if lv >= 0:
                _, i = read_long(i + 2, lv)
            else:
                while i < n and src[i] != "\n":
                    i += 1
            continue
        if c.isalpha() or c == "_":
            j = i
            while j < n and (src[j].isalnum() or src[j] == "_"):
                j += 1
            w = src[i:j]
            toks.append(Tok("kw" if w in _KEYWORDS else "name", w, line))
            i = j
            continue
        if c.isdigit() or (c == "." and i + 1 < n and src[i + 1].isdigit()):
            j = i
            if src.startswith(("0x", "0X"), i):
                j += 2
                while j < n and (src[j] in "0123456789abcdefABCDEF." or
                                 (src[j] in "pP") or (src[j] in "+-" and src[j - 1] in "pP")):
                    j += 1
            else:
                while j < n and (src[j].isdigit() or src[j] == "." or src[j] in "eE" or
                                 (src[j] in "+-" and src[j - 1] in "eE")):
                    j += 1
            v = str2number(src[i:j])
            if v is None:
                err(f"malformed number near '{src[i:j]}'")
            toks.append(Tok("number", v, line))
            i = j
            continue
        if c in "\"'":
            q = c
            j = i + 1
            out = []
            while True:
                if j >= n:
                    err("unfinished string")
                d = src[j]
                if d == q:
                    j += 1
                    break
                if d == "\n":
                    err("unfinished string")
                if d == "\\":
                    j += 1
                    e = src[j] if j < n else ""
                    if e in _ESC:
                        out.append(_ESC[e])
                        if e == "\n":
                            line += 1
                        j += 1
                    elif e == "x":
                        out.append(chr(int(src[j + 1:j + 3], 16)))
                        j += 3
                    elif e == "z":
                        j += 1
                        while j < n and src[j] in " \t\r\n":
                            if src[j] == "\n":
                                line += 1
                            j += 1
                    elif e.isdigit():
                        k = j
                        while k < n and k < j + 3 and src[k].isdigit():
                            k += 1
                        out.append(chr(int(src[j:k])))
                        j = k
                    elif e == "u":
                        k = src.index("}", j)
                        out.append(chr(int(src[j + 2:k], 16)))
                        j = k + 1
                    else:
                        err(f"invalid escape sequence '\\{e}'")
                else:
                    out.append(d)
                    j += 1
            toks.append(Tok("string", "".join(out), line))
            i = j
            continue
        if c == "[":
            lv = long_bracket(i)
            if lv >= 0:
                start_line = line
                body, i = read_long(i, lv)
                toks.append(Tok("string", body, start_line))
                continue
        for op in _OPS:
            if src.startswith(op, i):
                toks.append(Tok("op", op, line))
                i += len(op)
                break
        else:
            err(f"unexpected symbol near '{c}'")
    toks.append(Tok("eof", "<eof>", line))
    return toks


# ------------------------------------------------------------------------------------------ control flow
class _Break(Exception):
    pass


class _Return(Exception):
    __slots__ = ("vals",)

    def __init__(self, vals):
        self.vals = vals


class Scope:
    """A block's locals; closures keep their defining Scope, so upvalues are shared by reference."""
    __slots__ = ("vars", "parent", "varargs")

    def __init__(self, parent, varargs=None):
        self.vars = {}
        self.parent = parent
        self.varargs = varargs if varargs is not None else (parent.varargs if parent is not None else None)

    def find(self, name):
        s = self
        while s is not None:
            if name in s.vars:
                return s
            s = s.parent
        return None


# ------------------------------------------------------------------------------------------ parser/compiler
_BINPRI = {"or": (1, 1), "and": (2, 2), "<": (3, 3), ">": (3, 3), "<=": (3, 3), ">=": (3, 3), "~=": (3, 3),
           "==": (3, 3), "|": (4, 4), "~": (5, 5), "&": (6, 6), "<<": (7, 7), ">>": (7, 7), "..": (9, 8),
           "+": (10, 10), "-": (10, 10), "*": (11, 11), "/": (11, 11), "//": (11, 11), "%": (11, 11),
           "^": (14, 13)}
_UNARY_PRI = 12


class Compiler:
    """Recursive-descent parser that emits Python closures.

    Expressions compile to `f(scope) -> value`; a multi-value expression (call, `...`) also has a
    `.multi(scope) -> list` form. Statements compile to `f(scope) -> None`; `break` and `return`
    travel as exceptions.
    """

    def __init__(self, interp, toks, chunk):
        self.I = interp
        self.t = toks
        self.p = 0
        self.chunk = chunk

    # -- token helpers
    def peek(self, k=0):
        return self.t[self.p + k]

    def next(self):
        tok = self.t[self.p]
        self.p += 1
        return tok

    def check(self, kind, val=None):
        tok = self.t[self.p]
        return tok.kind == kind and (val is None or tok.val == val)

    def check_op(self, val):
        tok = self.t[self.p]
        return tok.kind == "op" and tok.val == val

    def check_kw(self, val):
        tok = self.t[self.p]
        return tok.kind == "kw" and tok.val == val

    def accept(self, kind, val):
        if self.check(kind, val):
            self.p += 1
            return True
        return False

    def expect(self, kind, val=None, what=None):
        tok = self.t[self.p]
        if tok.kind != kind or (val is not None and tok.val != val):
            want = val if val is not None else kind
            self.error(f"'{want}' expected near '{tok.val}'" if what is None else what, tok)
        self.p += 1
        return tok

    def error(self, msg, tok=None):
        tok = tok or self.t[self.p]
        raise LuaError(f"{self.chunk}:{tok.line}: {msg}")

    def where(self, tok):
        return f"{self.chunk}:{tok.line}:"

    # -- chunk / blocks
    def compile_chunk(self):
        body = self.block()
        if not self.check("eof"):
            self.error(f"'<eof>' expected near '{self.peek().val}'")
        return body

    def block_end(self):
        tok = self.peek()
        return tok.kind == "eof" or (tok.kind == "kw" and tok.val in ("end", "else", "elseif", "until"))

    def block(self):
        stmts = []
        while not self.block_end():
            if self.check_kw("return"):
                stmts.append(self.return_stat())
                break
            s = self.statement()
            if s is not None:
                stmts.append(s)
        stmts = tuple(stmts)
        if len(stmts) == 1:
            return stmts[0]

        def run(sc):
            for s in stmts:
                s(sc)
        return run

    def return_stat(self):
        self.next()
        if self.block_end() or self.check_op(";"):
            self.accept("op", ";")

            def ret0(sc):
                raise _Return([])
            return ret0
        exps = self.explist()
        self.accept("op", ";")
        ev = self.multi_list(exps)

        def ret(sc):
            raise _Return(ev(sc))
        return ret

    def statement(self):
        tok = self.peek()
        if tok.kind == "op" and tok.val == ";":
            self.next()
            return None
        if tok.kind == "kw":
            v = tok.val
            if v == "if":
                return self.if_stat()
            if v == "while":
                return self.while_stat()
            if v == "do":
                self.next()
                b = self.block()
                self.expect("kw", "end")

                def do(sc):
                    b(Scope(sc))
                return do
            if v == "for":
                return self.for_stat()
            if v == "repeat":
                return self.repeat_stat()
            if v == "function":
                return self.function_stat()
            if v == "local":
                self.next()
                if self.accept("kw", "function"):
                    return self.local_function()
                return self.local_stat()
            if v == "break":
                self.next()

                def brk(sc):
                    raise _Break()
                return brk
            if v == "goto":
                self.error("goto is not supported")
        if tok.kind == "op" and tok.val == "::":
            self.error("labels are not supported")
        return self.expr_stat()

    def if_stat(self):
        self.next()
        conds = []
        cond = self.expr()
        self.expect("kw", "then")
        conds.append((cond, self.block()))
        els = None
        while True:
            if self.accept("kw", "elseif"):
                c = self.expr()
                self.expect("kw", "then")
                conds.append((c, self.block()))
            elif self.accept("kw", "else"):
                els = self.block()
                self.expect("kw", "end")
                break
            else:
                self.expect("kw", "end")
                break
        conds = tuple(conds)

        def run(sc):
            for c, b in conds:
                v = c(sc)
                if v is not None and v is not False:
                    b(Scope(sc))
                    return
            if els is not None:
                els(Scope(sc))
        return run

    def while_stat(self):
        self.next()
        cond = self.expr()
        self.expect("kw", "do")
        body = self.block()
        self.expect("kw", "end")
        I = self.I

        def run(sc):
            try:
                while True:
                    v = cond(sc)
                    if v is None or v is False:
                        break
                    I.tick()
                    body(Scope(sc))
            except _Break:
                pass
        return run

    def repeat_stat(self):
        self.next()
        body = self.block()
        self.expect("kw", "until")
        cond = self.expr()
        I = self.I

        def run(sc):
            try:
                while True:
                    inner = Scope(sc)
                    I.tick()
                    body(inner)
                    v = cond(inner)  # the condition sees the body's locals
                    if v is not None and v is not False:
                        break
            except _Break:
                pass
        return run

    def for_stat(self):
        self.next()
        name1 = self.expect("name").val
        if self.accept("op", "="):
            e1 = self.expr()
            self.expect("op", ",")
            e2 = self.expr()
            e3 = self.expr() if self.accept("op", ",") else None
            self.expect("kw", "do")
            body = self.block()
            self.expect("kw", "end")
            I = self.I
            line = self.peek().line

            def run(sc):
                a, b = e1(sc), e2(sc)
                st = e3(sc) if e3 is not None else 1
                an, bn, sn = tonum(a), tonum(b), tonum(st)
                if an is None or bn is None or sn is None:
                    raise LuaError(f"{self.chunk}:{line}: 'for' initial value must be a number")
                if sn == 0:
                    raise LuaError(f"{self.chunk}:{line}: 'for' step is zero")
                try:
                    if type(an) is int and type(sn) is int:
                        if type(bn) is float:
                            bn = math.floor(bn) if sn > 0 else math.ceil(bn)
                        i = an
                        while (i <= bn) if sn > 0 else (i >= bn):
                            I.tick()
                            inner = Scope(sc)
                            inner.vars[name1] = i
                            body(inner)
                            i += sn
                    else:
                        i, bn, sn = float(an), float(bn), float(sn)
                        while (i <= bn) if sn > 0 else (i >= bn):
                            I.tick()
                            inner = Scope(sc)
                            inner.vars[name1] = i
                            body(inner)
                            i += sn
                except _Break:
                    pass
            return run
        names = [name1]
        while self.accept("op", ","):
            names.append(self.expect("name").val)
        self.expect("kw", "in")
        exps = self.multi_list(self.explist())
        self.expect("kw", "do")
        body = self.block()
        self.expect("kw", "end")
        I = self.I
        names = tuple(names)

        def run(sc):
            vals = exps(sc) + [None, None, None]
            f, s, ctl = vals[0], vals[1], vals[2]
            try:
                while True:
                    r = I.call(f, [s, ctl])
                    v0 = r[0] if r else None
                    if v0 is None:
                        break
                    ctl = v0
                    I.tick()
                    inner = Scope(sc)
                    for k, nm in enumerate(names):
                        inner.vars[nm] = r[k] if k < len(r) else None
                    body(inner)
            except _Break:
                pass
        return run

    def funcbody(self, name, is_method=False):
        line = self.peek().line
        self.expect("op", "(")
        params = ["self"] if is_method else []
        vararg = False
        if not self.check_op(")"):
            while True:
                if self.accept("op", "..."):
                    vararg = True
                    break
                params.append(self.expect("name").val)
                if not self.accept("op", ","):
                    break
        self.expect("op", ")")
        body = self.block()
        self.expect("kw", "end")
        params = tuple(params)
        I = self.I
        chunk = self.chunk

        def make(sc):
            def call(args):
                inner = Scope(sc, varargs=list(args[len(params):]) if vararg else [])
                v = inner.vars
                for k, p in enumerate(params):
                    v[p] = args[k] if k < len(args) else None
                I.depth += 1
                if I.depth > 190:
                    I.depth = 0
                    raise LuaError(f"{chunk}:{line}: stack overflow")
                try:
                    body(inner)
                except _Return as r:
                    return r.vals
                finally:
                    I.depth -= 1
                return []
            return LuaFunction(name, call)
        return make

    def function_stat(self):
        self.next()
        tok = self.expect("name")
        path = [tok.val]
        method = False
        while self.check_op(".") or self.check_op(":"):
            sep = self.next().val
            path.append(self.expect("name").val)
            if sep == ":":
                method = True
                break
        make = self.funcbody(".".join(path), is_method=method)
        I = self.I
        if len(path) == 1:
            nm = path[0]

            def run(sc):
                f = make(sc)
                s = sc.find(nm)
                if s is not None:
                    s.vars[nm] = f
                else:
                    I.globals.rawset(nm, f)
            return run
        head, keys, last = path[0], path[1:-1], path[-1]

        def run(sc):
            s = sc.find(head)
            obj = s.vars[head] if s is not None else I.globals.rawget(head)
            for k in keys:
                obj = I.index(obj, k)
            I.setindex(obj, last, make(sc))
        return run

    def local_function(self):
        nm = self.expect("name").val
        make = self.funcbody(nm)

        def run(sc):
            sc.vars[nm] = None
            sc.vars[nm] = make(sc)  # visible inside its own body (recursion)
        return run

    def local_stat(self):
        names = []
        while True:
            names.append(self.expect("name").val)
            if self.accept("op", "<"):  # attribs <const>/<close>
                self.expect("name")
                self.expect("op", ">")
            if not self.accept("op", ","):
                break
        if self.accept("op", "="):
            ev = self.multi_list(self.explist())
        else:
            ev = None
        names = tuple(names)
        if len(names) == 1 and ev is not None:
            nm = names[0]

            def run1(sc):
                vals = ev(sc)
                sc.vars[nm] = vals[0] if vals else None
            return run1

        def run(sc):
            vals = ev(sc) if ev is not None else []
            for k, nm in enumerate(names):
                sc.vars[nm] = vals[k] if k < len(vals) else None
        return run

    def expr_stat(self):
        tok = self.peek()
        target = self.suffixed_expr()
        if self.check_op("=") or self.check_op(","):
            targets = [target]
            while self.accept("op", ","):
                targets.append(self.suffixed_expr())
            self.expect("op", "=")
            ev = self.multi_list(self.explist())
            setters = []
            for t in targets:
                if t.kind not in ("name", "index"):
                    self.error("syntax error near '='", tok)
                setters.append(t.setter)
            setters = tuple(setters)
            if len(setters) == 1:
                s0 = setters[0]

                def assign1(sc):
                    vals = ev(sc)
                    s0(sc, vals[0] if vals else None)
                return assign1

            def assign(sc):
                vals = ev(sc)
                for k, s in enumerate(setters):
                    s(sc, vals[k] if k < len(vals) else None)
            return assign
        if target.kind != "call":
            self.error("syntax error near '%s'" % self.peek().val, tok)
        f = target.multi

        def callstat(sc):
            f(sc)
        return callstat

    # -- expressions
    def explist(self):
        exps = [self.expr()]
        while self.accept("op", ","):
            exps.append(self.expr())
        return exps

    def multi_list(self, exps):
        """Evaluator of an expression list: all values of the last expression, one of the others."""
        exps = tuple(exps)
        last = exps[-1]
        firsts = exps[:-1]
        lastm = getattr(last, "multi", None)
        if lastm is None:
            if not firsts:
                return lambda sc: [last(sc)]
            return lambda sc: [e(sc) for e in exps]
        if not firsts:
            return lastm
        return lambda sc: [e(sc) for e in firsts] + lastm(sc)

    def expr(self, limit=0):
        tok = self.peek()
        if (tok.kind == "kw" and tok.val == "not") or (tok.kind == "op" and tok.val in ("-", "#", "~")):
            self.next()
            op = tok.val
            operand = self.expr(_UNARY_PRI)
            left = self.unary(op, operand, tok)
        else:
            left = self.simple_expr()
        while True:
            tok = self.peek()
            op = tok.val if tok.kind in ("op", "kw") else None
            pri = _BINPRI.get(op)
            if pri is None or pri[0] <= limit:
                break
            self.next()
            right = self.expr(pri[1])
            left = self.binary(op, left, right, tok)
        return left

    def unary(self, op, e, tok):
        I = self.I
        where = self.where(tok)
        if op == "not":
            return _E(lambda sc: (lambda v: v is None or v is False)(e(sc)))
        if op == "-":
            if hasattr(e, "const"):
                v = e.const
                if type(v) in (int, float):
                    return _const(-v if type(v) is float else _wrap64(-v))
            return _E(lambda sc: I.arith("__unm", e(sc), None, where))
        if op == "#":
            return _E(lambda sc: I.length(e(sc), where))
        return _E(lambda sc: I.bitop("~", e(sc), None, where))

    def binary(self, op, a, b, tok):
        I = self.I
        where = self.where(tok)
        if op == "and":
            def f_and(sc):
                v = a(sc)
                return b(sc) if v is not None and v is not False else v
            return _E(f_and)
        if op == "or":
            def f_or(sc):
                v = a(sc)
                return v if v is not None and v is not False else b(sc)
            return _E(f_or)
        if op == "+":
            def add(sc):
                x, y = a(sc), b(sc)
                tx, ty = type(x), type(y)
                if tx is int and ty is int:
                    return _wrap64(x + y)
                if (tx is float or tx is int) and (ty is float or ty is int):
                    return float(x) + float(y)
                return I.arith("__add", x, y, where)
            return _E(add)
        if op == "-":
            def sub(sc):
                x, y = a(sc), b(sc)
                tx, ty = type(x), type(y)
                if tx is int and ty is int:
                    return _wrap64(x - y)
                if (tx is float or tx is int) and (ty is float or ty is int):
                    return float(x) - float(y)
                return I.arith("__sub", x, y, where)
            return _E(sub)
        if op == "*":
            def mul(sc):
                x, y = a(sc), b(sc)
                tx, ty = type(x), type(y)
                if tx is int and ty is int:
                    return _wrap64(x * y)
                if (tx is float or tx is int) and (ty is float or ty is int):
                    return float(x) * float(y)
                return I.arith("__mul", x, y, where)
            return _E(mul)
        if op == "/":
            def div(sc):
                x, y = a(sc), b(sc)
                tx, ty = type(x), type(y)
                if (tx is float or tx is int) and (ty is float or ty is int):
                    return _fdiv(float(x), float(y))
                return I.arith("__div", x, y, where)
            return _E(div)
        if op in ("%", "^", "//"):
            ev = {"%": "__mod", "^": "__pow", "//": "__idiv"}[op]
            return _E(lambda sc: I.arith(ev, a(sc), b(sc), where))
        if op == "..":
            return _E(lambda sc: I.concat(a(sc), b(sc), where))
        if op == "==":
            return _E(lambda sc: I.equal(a(sc), b(sc)))
        if op == "~=":
            return _E(lambda sc: not I.equal(a(sc), b(sc)))
        if op == "<":
            return _E(lambda sc: I.less(a(sc), b(sc), where))
        if op == ">":
            return _E(lambda sc: I.less(b(sc), a(sc), where))
        if op == "<=":
            return _E(lambda sc: I.less_equal(a(sc), b(sc), where))
        if op == ">=":
            return _E(lambda sc: I.less_equal(b(sc), a(sc), where))
        return _E(lambda sc: I.bitop(op, a(sc), b(sc), where))

    def simple_expr(self):
        tok = self.peek()
        k = tok.kind
        if k == "number":
            self.next()
            return _const(tok.val)
        if k == "string":
            self.next()
            return _const(tok.val)
        if k == "kw":
            if tok.val == "nil":
                self.next()
                return _const(None)
            if tok.val == "true":
                self.next()
                return _const(True)
            if tok.val == "false":
                self.next()
                return _const(False)
            if tok.val == "function":
                self.next()
                make = self.funcbody("anonymous")
                return _E(make)
        if k == "op":
            if tok.val == "...":
                self.next()

                def va(sc):
                    v = sc.varargs
                    return v[0] if v else None
                e = _E(va)
                e.multi = lambda sc: list(sc.varargs or [])
                return e
            if tok.val == "{":
                return self.table_cons()
        return self.suffixed_expr()

    def primary_expr(self):
        tok = self.peek()
        if tok.kind == "name":
            self.next()
            return self.name_ref(tok.val)
        if tok.kind == "op" and tok.val == "(":
            self.next()
            e = self.expr()
            self.expect("op", ")")
            inner = e
            return _E(lambda sc: inner(sc), kind="paren")  # truncates to one value
        self.error(f"unexpected symbol near '{tok.val}'")

    def name_ref(self, nm):
        I = self.I
        G = I.globals

        def get(sc):
            s = sc
            while s is not None:
                v = s.vars
                if nm in v:
                    return v[nm]
                s = s.parent
            return G.hash.get(nm) if G.meta is None else I.index(G, nm)

        def setter(sc, val):
            s = sc.find(nm)
            if s is not None:
                s.vars[nm] = val
            else:
                I.setindex(G, nm, val)
        return _E(get, kind="name", setter=setter)

    def suffixed_expr(self):
        e = self.primary_expr()
        while True:
            tok = self.peek()
            if tok.kind == "op":
                v = tok.val
                if v == ".":
                    self.next()
                    key = self.expect("name").val
                    e = self.index_expr(e, _const(key))
                    continue
                if v == "[":
                    self.next()
                    ke = self.expr()
                    self.expect("op", "]")
                    e = self.index_expr(e, ke)
                    continue
                if v == ":":
                    self.next()
                    mname = self.expect("name").val
                    args = self.call_args()
                    e = self.method_call(e, mname, args, tok)
                    continue
                if v in ("(", "{"):
                    args = self.call_args()
                    e = self.call_expr(e, args, tok)
                    continue
            if tok.kind == "string":
                args = self.call_args()
                e = self.call_expr(e, args, tok)
                continue
            return e

    def index_expr(self, obj, key):
        I = self.I

        def get(sc):
            o = obj(sc)
            k = key(sc)
            if type(o) is LuaTable:
                v = o.hash.get(_key(k))
                if v is not None or o.meta is None:
                    return v
            return I.index(o, k)

        def setter(sc, val):
            I.setindex(obj(sc), key(sc), val)
        return _E(get, kind="index", setter=setter)

    def call_args(self):
        tok = self.peek()
        if tok.kind == "string":
            self.next()
            return self.multi_list([_const(tok.val)])
        if tok.kind == "op" and tok.val == "{":
            t = self.table_cons()
            return self.multi_list([t])
        self.expect("op", "(")
        if self.accept("op", ")"):
            return lambda sc: []
        exps = self.explist()
        self.expect("op", ")")
        return self.multi_list(exps)

    def call_expr(self, fe, args, tok):
        I = self.I
        where = self.where(tok)
        fname = _describe(fe)

        def multi(sc):
            f = fe(sc)
            a = args(sc)
            if type(f) is LuaFunction:
                return f.call(a)
            return I.call(f, a, where, fname)
        e = _E(lambda sc: (lambda r: r[0] if r else None)(multi(sc)), kind="call")
        e.multi = multi
        return e

    def method_call(self, oe, mname, args, tok):
        I = self.I
        where = self.where(tok)

        def multi(sc):
            o = oe(sc)
            f = I.index(o, mname)
            return I.call(f, [o] + args(sc), where, f"method '{mname}'")
        e = _E(lambda sc: (lambda r: r[0] if r else None)(multi(sc)), kind="call")
        e.multi = multi
        return e

    def table_cons(self):
        self.expect("op", "{")
        items = []  # ("p", None, value) positional, ("k", key, value) keyed, in source order
        while not self.check_op("}"):
            tok = self.peek()
            if tok.kind == "op" and tok.val == "[":
                self.next()
                ke = self.expr()
                self.expect("op", "]")
                self.expect("op", "=")
                items.append(("k", ke, self.expr()))
            elif tok.kind == "name" and self.peek(1).kind == "op" and self.peek(1).val == "=":
                self.next()
                self.next()
                items.append(("k", _const(tok.val), self.expr()))
            else:
                items.append(("p", None, self.expr()))
            if not (self.accept("op", ",") or self.accept("op", ";")):
                break
        self.expect("op", "}")
        items = tuple(items)
        last_multi = items and items[-1][0] == "p" and hasattr(items[-1][2], "multi")

        def make(sc):
            t = LuaTable()
            h = t.hash
            n = 1
            last = len(items) - 1
            for idx, (kind, ke, ve) in enumerate(items):
                if kind == "p":
                    if idx == last and last_multi:
                        for v in ve.multi(sc):
                            if v is not None:
                                h[n] = v
                            n += 1
                    else:
                        v = ve(sc)
                        if v is not None:
                            h[n] = v
                        n += 1
                else:
                    k = ke(sc)
                    v = ve(sc)
                    t.rawset(k, v)
            return t
        return _E(make)


def _E(f, kind="expr", setter=None):
    """Marks a compiled expression: a function of the scope with a kind, and optionally `.multi`
    (all values) and `.setter` (assignment target)."""
    f.kind = kind
    f.setter = setter
    return f


def _const(v):
    f = _E(lambda sc: v, kind="const")
    f.const = v
    return f


def _describe(e):
    return {"name": "global", "index": "field", "call": "call result"}.get(e.kind, "value")


def _fdiv(x, y):
    try:
        return x / y
    except ZeroDivisionError:
        if x == 0 or x != x:
            return math.nan
        return math.copysign(math.inf, x) * math.copysign(1.0, y)


# ------------------------------------------------------------------------------------------ interpreter
class Interpreter:
    """One Lua state: globals, the standard libraries, and the runtime operations."""

    def __init__(self, out=None, instruction_limit=200_000_000):
        import sys
        if sys.getrecursionlimit() < 20000:
            sys.setrecursionlimit(20000)  # each Lua call nests a few Python frames
        self.globals = LuaTable()
        self.string_meta = LuaTable()
        self.out = out if out is not None else print
        self.depth = 0
        self.ticks = 0
        self.limit = instruction_limit
        self._open_libs()

    def tick(self):
        self.ticks += 1
        if self.ticks > self.limit:
            raise LuaError("script exceeded the loop iteration limit (infinite loop?)")

    # -- loading
    def compile(self, src: str, chunk: str = "chunk"):
        toks = tokenize(src, chunk)
        comp = Compiler(self, toks, chunk)
        body = comp.compile_chunk()

        def call(args):
            sc = Scope(None, varargs=list(args))
            try:
                body(sc)
            except _Return as r:
                return r.vals
            except _Break:
                raise LuaError(f"{chunk}: break outside a loop")
            return []
        return LuaFunction(chunk, call)

    def execute(self, src: str, chunk: str = "chunk", args=()):
        f = self.compile(src, chunk)
        return self.call(f, list(args))

    # -- metamethod helpers
    def metatable(self, v):
        if type(v) is LuaTable:
            return v.meta
        if type(v) is str:
            return self.string_meta
        return None

    def metamethod(self, v, event):
        m = self.metatable(v)
        return m.rawget(event) if m is not None else None

    def call(self, f, args, where="", what="value"):
        if type(f) is LuaFunction:
            return f.call(args)
        h = self.metamethod(f, "__call")
        if h is not None:
            return self.call(h, [f] + list(args), where)
        raise LuaError(f"{where} attempt to call a {lua_type(f)} value ({what})".strip())

    def index(self, o, k):
        for _ in range(100):
            if type(o) is LuaTable:
                v = o.hash.get(_key(k))
                if v is not None:
                    return v
                m = o.meta
                if m is None:
                    return None
                h = m.hash.get("__index")
                if h is None:
                    return None
            else:
                h = self.metamethod(o, "__index")
                if h is None:
                    raise LuaError(f"attempt to index a {lua_type(o)} value"
                                   + (f" (field '{k}')" if isinstance(k, str) else ""))
            if type(h) is LuaFunction:
                r = h.call([o, k])
                return r[0] if r else None
            o = h
        raise LuaError("'__index' chain too long; possible loop")

    def setindex(self, o, k, v):
        for _ in range(100):
            if type(o) is LuaTable:
                kk = _key(k)
                if kk in o.hash or o.meta is None:
                    o.rawset(k, v)
                    return
                h = o.meta.hash.get("__newindex")
                if h is None:
                    o.rawset(k, v)
                    return
            else:
                h = self.metamethod(o, "__newindex")
                if h is None:
                    raise LuaError(f"attempt to index a {lua_type(o)} value"
                                   + (f" (field '{k}')" if isinstance(k, str) else ""))
            if type(h) is LuaFunction:
                h.call([o, k, v])
                return
            o = h
        raise LuaError("'__newindex' chain too long; possible loop")

    def arith(self, event, a, b, where=""):
        if event == "__unm":
            x = tonum(a)
            if x is not None:
                return _wrap64(-x) if type(x) is int else -x
            h = self.metamethod(a, "__unm")
            if h is not None:
                r = self.call(h, [a, a])
                return r[0] if r else None
            raise LuaError(f"{where} attempt to perform arithmetic on a {lua_type(a)} value".strip())
        x, y = tonum(a), tonum(b)
        if x is not None and y is not None:
            return _arith_num(event, x, y)
        h = self.metamethod(a, event)
        if h is None:
            h = self.metamethod(b, event)
        if h is not None:
            r = self.call(h, [a, b])
            return r[0] if r else None
        bad = a if x is None else b
        raise LuaError(f"{where} attempt to perform arithmetic on a {lua_type(bad)} value".strip())

    def bitop(self, op, a, b, where=""):
        x = toint(a)
        y = toint(b) if op != "~" or b is not None else 0
        if x is None or y is None:
            ev = {"&": "__band", "|": "__bor", "~": "__bxor" if b is not None else "__bnot", "<<": "__shl",
                  ">>": "__shr"}[op]
            h = self.metamethod(a, ev) or self.metamethod(b, ev)
            if h is not None:
                r = self.call(h, [a, b])
                return r[0] if r else None
            raise LuaError(f"{where} number has no integer representation".strip())
        if op == "~" and b is None:
            return _wrap64(~x)
        if op == "&":
            return _wrap64(x & y)
        if op == "|":
            return _wrap64(x | y)
        if op == "~":
            return _wrap64(x ^ y)
        ux = x & 0xFFFFFFFFFFFFFFFF
        if op == "<<":
            return _wrap64(ux << y) if 0 <= y < 64 else (_wrap64(ux >> -y) if -64 < y < 0 else 0)
        return _wrap64(ux >> y) if 0 <= y < 64 else (_wrap64(ux << -y) if -64 < y < 0 else 0)

    def concat(self, a, b, where=""):
        ta, tb = type(a), type(b)
        if (ta is str or ta is int or ta is float) and (tb is str or tb is int or tb is float):
            return tostr(a) + tostr(b)
        h = self.metamethod(a, "__concat") or self.metamethod(b, "__concat")
        if h is not None:
            r = self.call(h, [a, b])
            return r[0] if r else None
        bad = b if (ta is str or ta is int or ta is float) else a
        raise LuaError(f"{where} attempt to concatenate a {lua_type(bad)} value".strip())

    def length(self, v, where=""):
        if type(v) is str:
            return len(v.encode("utf-8"))
        h = self.metamethod(v, "__len")
        if h is not None:
            r = self.call(h, [v])
            return r[0] if r else None
        if type(v) is LuaTable:
            return v.length()
        raise LuaError(f"{where} attempt to get length of a {lua_type(v)} value".strip())

    def equal(self, a, b):
        if a is b:
            return True
        ta, tb = type(a), type(b)
        if (ta is int or ta is float) and (tb is int or tb is float):
            return a == b
        if ta is bool or tb is bool:
            return ta is tb and a == b
        if ta is not tb:
            return False
        if ta is str:
            return a == b
        if ta is LuaTable:
            h = self.metamethod(a, "__eq") or self.metamethod(b, "__eq")
            if h is not None:
                r = self.call(h, [a, b])
                v = r[0] if r else None
                return v is not None and v is not False
        return False

    def less(self, a, b, where=""):
        ta, tb = type(a), type(b)
        if (ta is int or ta is float) and (tb is int or tb is float):
            return a < b
        if ta is str and tb is str:
            return a < b
        h = self.metamethod(a, "__lt") or self.metamethod(b, "__lt")
        if h is not None:
            r = self.call(h, [a, b])
            v = r[0] if r else None
            return v is not None and v is not False
        raise LuaError(f"{where} attempt to compare {_cmp_types(a, b)}".strip())

    def less_equal(self, a, b, where=""):
        ta, tb = type(a), type(b)
        if (ta is int or ta is float) and (tb is int or tb is float):
            return a <= b
        if ta is str and tb is str:
            return a <= b
        h = self.metamethod(a, "__le") or self.metamethod(b, "__le")
        if h is not None:
            r = self.call(h, [a, b])
            v = r[0] if r else None
            return v is not None and v is not False
        raise LuaError(f"{where} attempt to compare {_cmp_types(a, b)}".strip())

    def register(self, name, fn, table=None):
        """Exposes a Python function `fn(*args) -> value | tuple | None` as a Lua function."""
        def call(args):
            r = fn(*args)
            if r is None:
                return []
            if type(r) is tuple:
                return list(r)
            return [r]
        f = LuaFunction(name, call)
        (table or self.globals).rawset(name.split(".")[-1], f)
        return f

    # -- standard libraries
    def _open_libs(self):
        G = self.globals
        I = self
        G.rawset("_G", G)
        G.rawset("_VERSION", "Lua 5.4")

        def l_print(*args):
            I.out("\t".join(tostr(a, I) for a in args))
        self.register("print", l_print)
        self.register("type", lambda *a: lua_type(a[0]) if a else _argerr(1, "type", "value expected"))
        self.register("tostring", lambda v=None, *r: tostr(v, I))

        def l_tonumber(v=None, base=None, *r):
            if base is None:
                return (tonum(v) if type(v) in (int, float) else (str2number(v) if type(v) is str else None),)
            s = str(v).strip().lower()
            try:
                return (int(s, int(base)),)
            except ValueError:
                return (None,)
        self.register("tonumber", l_tonumber)

        def ipairs_step(args):
            i = args[1] + 1
            v = I.index(args[0], i)
            return [None] if v is None else [i, v]
        ipairs_iter = LuaFunction("ipairs_iter", ipairs_step)
        self.register("ipairs", lambda t=None, *r: (ipairs_iter, t, 0))

        def l_next(t, k=None, *r):
            keys = list(t.hash.keys())
            if k is None:
                idx = 0
            else:
                try:
                    idx = keys.index(_key(k)) + 1
                except ValueError:
                    raise LuaError("invalid key to 'next'")
            if idx >= len(keys):
                return (None,)
            kk = keys[idx]
            return (_unkey(kk), t.hash[kk])
        self.register("next", l_next)

        def l_pairs(t=None, *r):
            h = self.metamethod(t, "__pairs")
            if h is not None:
                res = self.call(h, [t])
                return tuple((res + [None, None, None])[:3])
            if type(t) is not LuaTable:
                raise LuaError(f"bad argument #1 to 'pairs' (table expected, got {lua_type(t)})")
            snapshot = list(t.hash.items())
            pos = {"i": 0}

            def it(args):
                while pos["i"] < len(snapshot):
                    kk, _ = snapshot[pos["i"]]
                    pos["i"] += 1
                    v = t.hash.get(kk)
                    if v is not None:
                        return [_unkey(kk), v]
                return [None]
            return (LuaFunction("pairs_iter", it), t, None)
        self.register("pairs", l_pairs)

        def l_select(n, *args):
            if n == "#":
                return len(args)
            n = toint(n)
            if n is None:
                raise LuaError("bad argument #1 to 'select' (number expected)")
            if n < 0:
                n = len(args) + n + 1
                if n < 1:
                    raise LuaError("bad argument #1 to 'select' (index out of range)")
            return tuple(args[n - 1:])
        self.register("select", l_select)

        def l_error(msg=None, level=1, *r):
            raise LuaError(msg)
        self.register("error", l_error)

        def l_assert(v=None, msg="assertion failed!", *rest):
            if v is None or v is False:
                raise LuaError(msg)
            return (v, msg) + rest
        self.register("assert", l_assert)

        def l_pcall(f, *args):
            depth = I.depth
            try:
                return tuple([True] + I.call(f, list(args)))
            except LuaError as e:
                I.depth = depth
                return (False, e.value)
            except RecursionError:
                I.depth = depth
                return (False, "stack overflow")
        self.register("pcall", l_pcall)

        def l_setmetatable(t, m=None, *r):
            if type(t) is not LuaTable:
                raise LuaError("bad argument #1 to 'setmetatable' (table expected)")
            if t.meta is not None and t.meta.rawget("__metatable") is not None:
                raise LuaError("cannot change a protected metatable")
            t.meta = m
            return t
        self.register("setmetatable", l_setmetatable)

        def l_getmetatable(v=None, *r):
            m = I.metatable(v)
            if m is None:
                return (None,)
            p = m.rawget("__metatable")
            return p if p is not None else m
        self.register("getmetatable", l_getmetatable)
        self.register("rawget", lambda t, k=None, *r: (t.rawget(k),))
        self.register("rawset", lambda t, k, v=None, *r: (t.rawset(k, v), t)[1])
        self.register("rawequal", lambda a=None, b=None, *r: a is b or (type(a) is type(b) and a == b
                                                                           and type(a) is not LuaTable))
        self.register("rawlen", lambda v, *r: v.length() if type(v) is LuaTable else len(v))

        def l_load(chunk, name="=(load)", mode="bt", env=None, *r):
            if not isinstance(chunk, str):
                return (None, "load: only text chunks are supported")
            try:
                return I.compile(chunk, str(name).lstrip("=@"))
            except LuaError as e:
                return (None, e.value)
        self.register("load", l_load)

        # string
        S = LuaTable()
        G.rawset("string", S)
        self.string_meta.rawset("__index", S)
        self.register("format", lambda fmt, *a: lua_format(I, fmt, a), S)
        self.register("rep", lambda s, n, sep="", *r: sep.join([tostr(s)] * max(0, toint(n) or 0)), S)
        self.register("upper", lambda s, *r: tostr(s).upper(), S)
        self.register("lower", lambda s, *r: tostr(s).lower(), S)
        self.register("len", lambda s, *r: len(tostr(s)), S)
        self.register("reverse", lambda s, *r: tostr(s)[::-1], S)

        def l_sub(s, i=1, j=-1, *r):
            s = tostr(s)
            n = len(s)
            i, j = toint(i), toint(j)
            if i < 0:
                i = max(n + i + 1, 1)
            elif i == 0:
                i = 1
            if j < 0:
                j = n + j + 1
            elif j > n:
                j = n
            return s[i - 1:j] if i <= j else ""
        self.register("sub", l_sub, S)

        def l_byte(s, i=1, j=None, *r):
            s = tostr(s)
            i = toint(i)
            j = i if j is None else toint(j)
            n = len(s)
            if i < 0:
                i = n + i + 1
            if j < 0:
                j = n + j + 1
            return tuple(ord(c) for c in s[max(i, 1) - 1:j])
        self.register("byte", l_byte, S)
        self.register("char", lambda *a: "".join(chr(toint(c)) for c in a), S)

        def l_find(s, pat, init=1, plain=False, *r):
            s, init = tostr(s), toint(init)
            if init < 0:
                init = max(len(s) + init + 1, 1)
            if plain or not any(c in pat for c in "^$*+?.([%-"):
                k = s.find(pat, init - 1)
                return (None,) if k < 0 else (k + 1, k + len(pat))
            m = _lua_pattern(pat).search(s, init - 1)
            if not m:
                return (None,)
            return (m.start() + 1, m.end()) + tuple(m.groups())
        self.register("find", l_find, S)

        def l_match(s, pat, init=1, *r):
            m = _lua_pattern(pat).search(tostr(s), max(toint(init), 1) - 1)
            if not m:
                return (None,)
            return tuple(m.groups()) if m.groups() else m.group(0)
        self.register("match", l_match, S)

        def l_gmatch(s, pat, *r):
            it = _lua_pattern(pat).finditer(tostr(s))

            def step(args):
                m = next(it, None)
                if m is None:
                    return [None]
                return list(m.groups()) if m.groups() else [m.group(0)]
            return LuaFunction("gmatch_iter", step)
        self.register("gmatch", l_gmatch, S)

        def l_gsub(s, pat, repl, n=None, *r):
            rx = _lua_pattern(pat)
            count = [0]
            limit = toint(n) if n is not None else -1

            def sub(m):
                if limit >= 0 and count[0] >= limit:
                    return m.group(0)
                count[0] += 1
                whole = m.group(0)
                caps = m.groups() or (whole,)
                if isinstance(repl, str):
                    return re.sub(r"%([0-9%])", lambda g: whole if g.group(1) == "0" else (
                        "%" if g.group(1) == "%" else tostr(caps[int(g.group(1)) - 1])), repl)
                if type(repl) is LuaTable:
                    v = I.index(repl, caps[0])
                else:
                    rr = I.call(repl, list(caps))
                    v = rr[0] if rr else None
                return whole if v is None or v is False else tostr(v)
            out = rx.sub(sub, tostr(s))
            return (out, count[0])
        self.register("gsub", l_gsub, S)

        # math
        M = LuaTable()
        G.rawset("math", M)
        M.rawset("pi", math.pi)
        M.rawset("huge", math.inf)
        M.rawset("maxinteger", (1 << 63) - 1)
        M.rawset("mininteger", -(1 << 63))

        def num(v, fname, k=1):
            x = tonum(v)
            if x is None:
                raise LuaError(f"bad argument #{k} to '{fname}' (number expected, got {lua_type(v)})")
            return x

        def l_floor(x, *r):
            x = num(x, "floor")
            if type(x) is int:
                return x
            f = math.floor(x) if math.isfinite(x) else x
            return int(f) if math.isfinite(x) and -(1 << 63) <= f < (1 << 63) else float(f)
        self.register("floor", l_floor, M)

        def l_ceil(x, *r):
            x = num(x, "ceil")
            if type(x) is int:
                return x
            f = math.ceil(x) if math.isfinite(x) else x
            return int(f) if math.isfinite(x) and -(1 << 63) <= f < (1 << 63) else float(f)
        self.register("ceil", l_ceil, M)
        self.register("abs", lambda x, *r: abs(num(x, "abs")), M)

        def l_max(*a):
            if not a:
                raise LuaError("bad argument #1 to 'max' (number expected, got no value)")
            best = num(a[0], "max")
            for k, v in enumerate(a[1:], 2):
                v = num(v, "max", k)
                if best < v:
                    best = v
            return best
        self.register("max", l_max, M)

        def l_min(*a):
            if not a:
                raise LuaError("bad argument #1 to 'min' (number expected, got no value)")
            best = num(a[0], "min")
            for k, v in enumerate(a[1:], 2):
                v = num(v, "min", k)
                if v < best:
                    best = v
            return best
        self.register("min", l_min, M)

        def fl(fn, name):
            def f(x, *r):
                try:
                    return fn(float(num(x, name)))
                except (ValueError, OverflowError):
                    return math.nan
            return f
        self.register("sqrt", fl(lambda x: math.sqrt(x) if x >= 0 else math.nan, "sqrt"), M)
        self.register("sin", fl(math.sin, "sin"), M)
        self.register("cos", fl(math.cos, "cos"), M)
        self.register("tan", fl(math.tan, "tan"), M)
        self.register("asin", fl(lambda x: math.asin(x) if -1 <= x <= 1 else math.nan, "asin"), M)
        self.register("acos", fl(lambda x: math.acos(x) if -1 <= x <= 1 else math.nan, "acos"), M)
        self.register("exp", fl(math.exp, "exp"), M)
        self.register("atan", lambda y, x=1.0, *r: math.atan2(float(num(y, "atan")), float(num(x, "atan", 2))), M)
        self.register("deg", lambda x, *r: float(num(x, "deg")) * (180.0 / math.pi), M)
        self.register("rad", lambda x, *r: float(num(x, "rad")) * (math.pi / 180.0), M)

        def l_log(x, base=None, *r):
            x = float(num(x, "log"))
            try:
                if base is None:
                    return math.log(x) if x > 0 else (-math.inf if x == 0 else math.nan)
                b = float(num(base, "log", 2))
                if b == 2.0:
                    return math.log2(x)
                if b == 10.0:
                    return math.log10(x)
                return math.log(x) / math.log(b)
            except ValueError:
                return math.nan
        self.register("log", l_log, M)

        def l_fmod(a, b, *r):
            a, b = num(a, "fmod"), num(b, "fmod", 2)
            if type(a) is int and type(b) is int:
                if b == 0:
                    raise LuaError("bad argument #2 to 'fmod' (zero)")
                return int(math.fmod(a, b))
            return math.fmod(float(a), float(b))
        self.register("fmod", l_fmod, M)

        def l_modf(x, *r):
            x = float(num(x, "modf"))
            if math.isinf(x):
                return (x, 0.0)
            ip = float(math.trunc(x))
            return (ip if not ip.is_integer() else (int(ip) if abs(ip) < 2 ** 63 else ip), x - ip)
        self.register("modf", lambda x, *r: (lambda v: (float(v[0]), v[1]))(l_modf(x)), M)
        self.register("tointeger", lambda x=None, *r: (toint(x) if type(x) in (int, float) else None,), M)
        self.register("type", lambda x=None, *r: (("integer" if type(x) is int else "float")
                                                  if type(x) in (int, float) else None,), M)
        self.register("ult", lambda a, b, *r: (a & 0xFFFFFFFFFFFFFFFF) < (b & 0xFFFFFFFFFFFFFFFF), M)
        self.rng = Xoshiro256()
        self.rng.seed(0x5EED, 0)  # Lua seeds randomly; a fixed default keeps runs reproducible

        def l_random(m=None, n=None, *r):
            rv = self.rng.next()
            if m is None:
                return (rv >> 11) * (0.5 / (1 << 52))
            lo, hi = (1, toint(m)) if n is None else (toint(m), toint(n))
            if lo is None or hi is None:
                raise LuaError("bad argument to 'random' (number has no integer representation)")
            if lo > hi:
                raise LuaError("bad argument to 'random' (interval is empty)")
            return lo + self.rng.project(rv, (hi - lo) & 0xFFFFFFFFFFFFFFFF)
        self.register("random", l_random, M)

        def l_randomseed(n1=None, n2=0, *r):
            if n1 is None:
                self.rng.seed(0x5EED, 0)
                return None
            v = n1 if type(n1) is int else _float_to_seed(float(n1))
            self.rng.seed(v, toint(n2) or 0)
            return None
        self.register("randomseed", l_randomseed, M)

        # table
        T = LuaTable()
        G.rawset("table", T)

        def l_insert(t, *a):
            n = t.length()
            if len(a) == 1:
                t.rawset(n + 1, a[0])
            elif len(a) == 2:
                pos = toint(a[0])
                if pos < 1 or pos > n + 1:
                    raise LuaError("bad argument #2 to 'insert' (position out of bounds)")
                for i in range(n, pos - 1, -1):
                    t.rawset(i + 1, t.rawget(i))
                t.rawset(pos, a[1])
            else:
                raise LuaError("wrong number of arguments to 'insert'")
        self.register("insert", l_insert, T)

        def l_remove(t, pos=None, *r):
            n = t.length()
            if pos is None:
                pos = n
            pos = toint(pos)
            if n == 0 and pos in (0, n):
                return t.rawget(pos)
            v = t.rawget(pos)
            for i in range(pos, n):
                t.rawset(i, t.rawget(i + 1))
            t.rawset(n, None)
            return v
        self.register("remove", l_remove, T)

        def l_concat(t, sep="", i=1, j=None, *r):
            j = t.length() if j is None else toint(j)
            return tostr(sep).join(tostr(t.rawget(k)) for k in range(toint(i), j + 1))
        self.register("concat", l_concat, T)

        def l_unpack(t, i=1, j=None, *r):
            j = t.length() if j is None else toint(j)
            return tuple(I.index(t, k) for k in range(toint(i), j + 1))
        self.register("unpack", l_unpack, T)
        G.rawset("unpack", T.rawget("unpack"))

        def l_pack(*a):
            t = LuaTable(list(a))
            t.rawset("n", len(a))
            return t
        self.register("pack", l_pack, T)

        def l_sort(t, comp=None, *r):
            import functools
            arr = t.array()
            if comp is None:
                key = functools.cmp_to_key(lambda a, b: -1 if I.less(a, b) else (1 if I.less(b, a) else 0))
            else:
                def cmpf(a, b):
                    if _truthy(I.call(comp, [a, b])):
                        return -1
                    if _truthy(I.call(comp, [b, a])):
                        return 1
                    return 0
                key = functools.cmp_to_key(cmpf)
            arr.sort(key=key)
            for k, v in enumerate(arr, 1):
                t.rawset(k, v)
        self.register("sort", l_sort, T)

        # os (clock/time only)
        O = LuaTable()
        G.rawset("os", O)
        import time as _time
        self.register("clock", lambda *a: _time.process_time(), O)
        self.register("time", lambda *a: int(_time.time()), O)


def _truthy(r):
    v = r[0] if r else None
    return v is not None and v is not False


def _argerr(k, fname, msg):
    raise LuaError(f"bad argument #{k} to '{fname}' ({msg})")


def _cmp_types(a, b):
    ta, tb = lua_type(a), lua_type(b)
    return f"two {ta} values" if ta == tb else f"{ta} with {tb}"


def _arith_num(event, x, y):
    if event == "__add":
        return _wrap64(x + y) if type(x) is int and type(y) is int else float(x) + float(y)
    if event == "__sub":
        return _wrap64(x - y) if type(x) is int and type(y) is int else float(x) - float(y)
    if event == "__mul":
        return _wrap64(x * y) if type(x) is int and type(y) is int else float(x) * float(y)
    if event == "__div":
        return _fdiv(float(x), float(y))
    if event == "__pow":
        try:
            return math.pow(float(x), float(y))
        except (OverflowError, ValueError):
            return math.inf if float(x) > 0 else math.nan
    if event == "__idiv":
        if type(x) is int and type(y) is int:
            if y == 0:
                raise LuaError("attempt to perform 'n//0'")
            return x // y
        q = _fdiv(float(x), float(y))
        return math.floor(q) * 1.0 if math.isfinite(q) else q
    if event == "__mod":
        if type(x) is int and type(y) is int:
            if y == 0:
                raise LuaError("attempt to perform 'n%%0'")
            return x % y
        x, y = float(x), float(y)
        if y == 0:
            return math.nan
        if math.isinf(y):
            return x if (x >= 0) == (y > 0) or x == 0 else y
        m = math.fmod(x, y)
        if m != 0 and (m < 0) != (y < 0):
            m += y
        return m
    raise LuaError(f"bad arithmetic event {event}")


def _float_to_seed(x: float) -> int:
    """Lua 5.4 math.randomseed with a float argument: the float's value cast to an integer."""
    if x.is_integer() and -(1 << 63) <= x < (1 << 63):
        return int(x)
    return struct.unpack("<q", struct.pack("<d", x))[0]


class Xoshiro256:
    """xoshiro256** (Blackman and Vigna) with Lua 5.4's seeding and interval projection."""

    M = 0xFFFFFFFFFFFFFFFF

    def __init__(self):
        self.s = [0, 0, 0, 0]

    @staticmethod
    def _rotl(x, n):
        return ((x << n) | (x >> (64 - n))) & Xoshiro256.M

    def next(self):
        s = self.s
        s0, s1, s2, s3 = s
        s2 ^= s0
        s3 ^= s1
        res = (self._rotl((s1 * 5) & self.M, 7) * 9) & self.M
        s1 ^= s2
        s0 ^= s3
        s2 ^= (s[1] << 17) & self.M
        s3 = self._rotl(s3, 45)
        self.s = [s0, s1, s2, s3]
        return res

    def seed(self, n1: int, n2: int):
        self.s = [n1 & self.M, 0xFF, n2 & self.M, 0]
        for _ in range(16):
            self.next()  # discard initial values to "spread" the seed

    def project(self, ran: int, n: int) -> int:
        """A value uniformly in [0, n] from `ran`, by rejection on the smallest covering bit mask."""
        if n & (n + 1) == 0:  # n + 1 is a power of two
            return ran & n
        lim = n
        lim |= lim >> 1
        lim |= lim >> 2
        lim |= lim >> 4
        lim |= lim >> 8
        lim |= lim >> 16
        lim |= lim >> 32
        while True:
            ran &= lim
            if ran <= n:
                return ran
            ran = self.next()


# ------------------------------------------------------------------------------------------ string.format
_FMT = re.compile(r"%([-+ #0]*)(\d*)(?:\.(\d+))?([diouxXeEfgGqscaA%])")


def lua_format(interp, fmt, args):
    fmt = tostr(fmt)
    out = []
    pos = 0
    ai = 0
    for m in _FMT.finditer(fmt):
        out.append(fmt[pos:m.start()])
        pos = m.end()
        flags, width, prec, conv = m.groups()
        if conv == "%":
            out.append("%")
            continue
        if ai >= len(args):
            raise LuaError(f"bad argument #{ai + 2} to 'format' (no value)")
        v = args[ai]
        ai += 1
        spec = "%" + flags + width + (("." + prec) if prec is not None else "")
        if conv in "di":
            iv = toint(v)
            if iv is None:
                raise LuaError(f"bad argument #{ai + 1} to 'format' (number has no integer representation)")
            out.append((spec + "d") % iv)
        elif conv in "ouxX":
            iv = toint(v)
            if iv is None:
                raise LuaError(f"bad argument #{ai + 1} to 'format' (number has no integer representation)")
            out.append((spec + conv) % (iv & 0xFFFFFFFFFFFFFFFF if iv < 0 else iv))
        elif conv in "eEfgG":
            x = tonum(v)
            if x is None:
                raise LuaError(f"bad argument #{ai + 1} to 'format' (number expected, got {lua_type(v)})")
            s = (spec + conv) % float(x)
            out.append(s.replace("inf", "inf").replace("nan", "nan" if float(x) == float(x) else "nan"))
        elif conv in "aA":
            out.append(float(tonum(v)).hex())
        elif conv == "c":
            out.append(chr(toint(v)))
        elif conv == "s":
            s = tostr(v, interp)
            out.append((spec + "s") % s)
        elif conv == "q":
            if isinstance(v, str):
                out.append('"' + v.replace("\\", "\\\\").replace('"', '\\"').replace("\n", "\\n") + '"')
            else:
                out.append(tostr(v))
    out.append(fmt[pos:])
    return "".join(out)


# ------------------------------------------------------------------------------------------ patterns
_CLASSES = {"a": "A-Za-z", "d": "0-9", "l": "a-z", "s": r" \t\n\r\f\v", "u": "A-Z", "w": "A-Za-z0-9",
            "x": "A-Fa-f0-9", "p": r"!-/:-@\[-`{-~", "c": r"\x00-\x1f\x7f"}


def _lua_pattern(pat: str):
    """Translates the common subset of Lua patterns to a Python regex."""
    out = []
    i, n = 0, len(pat)
    while i < n:
        c = pat[i]
        if c == "%":
            i += 1
            d = pat[i]
            if d.lower() in _CLASSES:
                cls = _CLASSES[d.lower()]
                out.append(f"[^{cls}]" if d.isupper() else f"[{cls}]")
            else:
                out.append(re.escape(d))
        elif c == "[":
            j = i + 1
            buf = ["["]
            if j < n and pat[j] == "^":
                buf.append("^")
                j += 1
            first = True
            while j < n and (pat[j] != "]" or first):
                first = False
                if pat[j] == "%":
                    d = pat[j + 1]
                    buf.append(_CLASSES.get(d.lower(), re.escape(d)) if d.lower() in _CLASSES else re.escape(d))
                    j += 2
                else:
                    buf.append("\\" + pat[j] if pat[j] in "\\^[" else pat[j])
                    j += 1
            buf.append("]")
            out.append("".join(buf))
            i = j
        elif c == "-":
            out.append("*?")
        elif c == "(" and i + 1 < n and pat[i + 1] == ")":
            out.append("()")
            i += 1
        elif c in "().*+?^$":
            out.append(c)
        else:
            out.append(re.escape(c))
        i += 1
    return re.compile("".join(out))
