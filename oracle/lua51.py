"""A small Lua 5.1 interpreter, enough to run the reference's build-time
code generators (lib/vla0.c.lua, lib/vlaw0.c.lua, include/vec_ops_c.h.lua
and the Complex/Matrix/Gamma modules they require) where no Lua is
installed.  Test infrastructure: it only produces the generated C sources
the reference's Makefiles would make with `lua script.lua > out`, so that
the reference can be compiled as a second oracle.

Covered: the whole Lua 5.1 syntax (locals, closures, varargs, multiple
assignment and returns, numeric and generic for, while, repeat, if,
method calls, table constructors, long strings and comments), numbers as
doubles printed with "%.14g", metatables (__index, __newindex, __call,
arithmetic, __unm, __concat, __eq, __lt, __le, __len, __tostring) and the
parts of the standard library code generators use (print, io.write,
string.*, table.*, math.*, pairs/ipairs/next, select, unpack, type,
tostring, tonumber, setmetatable/getmetatable, rawget/rawset/rawequal,
assert, error, pcall, require).

Usage: python lua51.py script.lua > out   (modules are looked up next to
the script, as Lua's default package.path './?.lua' does when run from the
script's directory).
"""
import math
import os
import re
import sys

# ------------------------------------------------------------------ lexer

_KEYWORDS = {"and", "break", "do", "else", "elseif", "end", "false", "for", "function", "if",
             "in", "local", "nil", "not", "or", "repeat", "return", "then", "true", "until",
             "while"}
_OPS3 = ("...",)
_OPS2 = ("==", "~=", "<=", ">=", "..")
_OPS1 = "+-*/%^#<>=(){}[];:,."


class LuaError(Exception):
    def __init__(self, value, where=""):
        super().__init__(value)
        self.value = value
        self.where = where


def _long_bracket(src, i):
    """at src[i] == '[': the level of a long bracket [==[ or -1"""
    j = i + 1
    while j < len(src) and src[j] == "=":
        j += 1
    if j < len(src) and src[j] == "[":
        return j - i - 1
    return -1


def _read_long(src, i, level, line):
    """reads a long string/comment starting at src[i] ('['); returns (text,
    index after it, new line)"""
    start = i + level + 2
    close = "]" + "="*level + "]"
    end = src.find(close, start)
    if end < 0:
        raise LuaError("unfinished long string/comment at line %d" % line)
    text = src[start:end]
    if text.startswith("\r\n"):
        text = text[2:]
    elif text.startswith("\n"):
        text = text[1:]
    return text, end + len(close), line + src.count("\n", i, end + len(close))


_ESC = {"n": "\n", "t": "\t", "r": "\r", "a": "\a", "b": "\b", "f": "\f", "v": "\v", "\\": "\\",
        '"': '"', "'": "'", "\n": "\n"}


def tokenize(src):
    toks = []
    i, n, line = 0, len(src), 1
    if src.startswith("#"):                          # shebang line
        i = src.find("\n")
        i = n if i < 0 else i
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
            if i + 2 < n and src[i + 2] == "[":
                lv = _long_bracket(src, i + 2)
                if lv >= 0:
                    _, i, line = _read_long(src, i + 2, lv, line)
                    continue
            j = src.find("\n", i)
            i = n if j < 0 else j
            continue
        if c.isalpha() or c == "_":
            j = i + 1
            while j < n and (src[j].isalnum() or src[j] == "_"):
                j += 1
            w = src[i:j]
            toks.append(("kw" if w in _KEYWORDS else "name", w, line))
            i = j
            continue
        if c.isdigit() or (c == "." and i + 1 < n and src[i + 1].isdigit()):
            m = re.compile(r"0[xX][0-9a-fA-F]+|(\d+\.?\d*|\.\d+)([eE][+-]?\d+)?").match(src, i)
            t = m.group(0)
            val = float(int(t, 16)) if t[:2].lower() == "0x" else float(t)
            toks.append(("num", val, line))
            i = m.end()
            continue
        if c in "\"'":
            j = i + 1
            buf = []
            while True:
                if j >= n:
                    raise LuaError("unfinished string at line %d" % line)
                d = src[j]
                if d == c:
                    j += 1
                    break
                if d == "\n":
                    raise LuaError("unfinished string at line %d" % line)
                if d == "\\":
                    e = src[j + 1]
                    if e in _ESC:
                        buf.append(_ESC[e])
                        if e == "\n":
                            line += 1
                        j += 2
                    elif e.isdigit():
                        k = j + 1
                        while k < n and k < j + 4 and src[k].isdigit():
                            k += 1
                        buf.append(chr(int(src[j + 1:k])))
                        j = k
                    else:
                        buf.append(e)
                        j += 2
                    continue
                buf.append(d)
                j += 1
            toks.append(("str", "".join(buf), line))
            i = j
            continue
        if c == "[":
            lv = _long_bracket(src, i)
            if lv >= 0:
                text, i, l2 = _read_long(src, i, lv, line)
                toks.append(("str", text, line))
                line = l2
                continue
        if src.startswith("...", i):
            toks.append(("op", "...", line))
            i += 3
            continue
        two = src[i:i + 2]
        if two in _OPS2:
            toks.append(("op", two, line))
            i += 2
            continue
        if c in _OPS1:
            toks.append(("op", c, line))
            i += 1
            continue
        raise LuaError("unexpected character %r at line %d" % (c, line))
    toks.append(("eof", None, line))
    return toks


# ----------------------------------------------------------------- parser
# AST nodes are tuples whose first element names the node.

_BINPRI = {"or": (1, 1), "and": (2, 2), "<": (3, 3), ">": (3, 3), "<=": (3, 3), ">=": (3, 3),
           "~=": (3, 3), "==": (3, 3), "..": (5, 4), "+": (6, 6), "-": (6, 6), "*": (7, 7),
           "/": (7, 7), "%": (7, 7), "^": (10, 9)}
_UNARY_PRI = 8


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

    def check(self, kind, val=None):
        tok = self.t[self.i]
        return tok[0] == kind and (val is None or tok[1] == val)

    def accept(self, kind, val=None):
        if self.check(kind, val):
            return self.next()
        return None

    def expect(self, kind, val=None):
        tok = self.next()
        if tok[0] != kind or (val is not None and tok[1] != val):
            raise LuaError("line %d: expected %s %s, got %s %r" % (tok[2], kind, val or "", tok[0],
                                                                     tok[1]))
        return tok

    def block_end(self):
        tok = self.peek()
        return tok[0] == "eof" or (tok[0] == "kw" and tok[1] in ("end", "else", "elseif", "until"))

    def block(self):
        stats = []
        while not self.block_end():
            if self.check("kw", "return"):
                line = self.next()[2]
                exps = []
                if not self.block_end() and not self.check("op", ";"):
                    exps = self.explist()
                self.accept("op", ";")
                stats.append(("return", exps, line))
                break
            if self.check("kw", "break"):
                self.next()
                self.accept("op", ";")
                stats.append(("break",))
                break
            st = self.statement()
            if st is not None:
                stats.append(st)
            self.accept("op", ";")
        return stats

    def statement(self):
        tok = self.peek()
        line = tok[2]
        if tok[0] == "op" and tok[1] == ";":
            self.next()
            return None
        if tok[0] == "kw":
            k = tok[1]
            if k == "do":
                self.next()
                b = self.block()
                self.expect("kw", "end")
                return ("do", b)
            if k == "while":
                self.next()
                cond = self.expr()
                self.expect("kw", "do")
                b = self.block()
                self.expect("kw", "end")
                return ("while", cond, b)
            if k == "repeat":
                self.next()
                b = self.block()
                self.expect("kw", "until")
                cond = self.expr()
                return ("repeat", b, cond)
            if k == "if":
                self.next()
                clauses = []
                cond = self.expr()
                self.expect("kw", "then")
                clauses.append((cond, self.block()))
                other = None
                while True:
                    if self.accept("kw", "elseif"):
                        cond = self.expr()
                        self.expect("kw", "then")
                        clauses.append((cond, self.block()))
                    elif self.accept("kw", "else"):
                        other = self.block()
                        self.expect("kw", "end")
                        break
                    else:
                        self.expect("kw", "end")
                        break
                return ("if", clauses, other)
            if k == "for":
                self.next()
                n1 = self.expect("name")[1]
                if self.accept("op", "="):
                    a = self.expr()
                    self.expect("op", ",")
                    b = self.expr()
                    c = self.expr() if self.accept("op", ",") else None
                    self.expect("kw", "do")
                    body = self.block()
                    self.expect("kw", "end")
                    return ("fornum", n1, a, b, c, body, line)
                names = [n1]
                while self.accept("op", ","):
                    names.append(self.expect("name")[1])
                self.expect("kw", "in")
                exps = self.explist()
                self.expect("kw", "do")
                body = self.block()
                self.expect("kw", "end")
                return ("forin", names, exps, body, line)
            if k == "function":
                self.next()
                target = ("name", self.expect("name")[1], line)
                is_method = False
                while self.check("op", ".") or self.check("op", ":"):
                    sep = self.next()[1]
                    key = self.expect("name")[1]
                    target = ("index", target, ("const", key), line)
                    if sep == ":":
                        is_method = True
                        break
                fn = self.funcbody(is_method, line)
                return ("assign", [target], [fn], line)
            if k == "local":
                self.next()
                if self.accept("kw", "function"):
                    name = self.expect("name")[1]
                    fn = self.funcbody(False, line)
                    return ("localfunc", name, fn)
                names = [self.expect("name")[1]]
                while self.accept("op", ","):
                    names.append(self.expect("name")[1])
                exps = self.explist() if self.accept("op", "=") else []
                return ("local", names, exps, line)
        # expression statement: assignment or call
        e = self.suffixedexp()
        if self.check("op", "=") or self.check("op", ","):
            targets = [e]
            while self.accept("op", ","):
                targets.append(self.suffixedexp())
            self.expect("op", "=")
            exps = self.explist()
            for t in targets:
                if t[0] not in ("name", "index"):
                    raise LuaError("line %d: cannot assign to this expression" % line)
            return ("assign", targets, exps, line)
        if e[0] not in ("call", "method"):
            raise LuaError("line %d: syntax error (expression is not a statement)" % line)
        return ("exprstat", e)

    def funcbody(self, is_method, line):
        self.expect("op", "(")
        params = ["self"] if is_method else []
        vararg = False
        if not self.check("op", ")"):
            while True:
                if self.accept("op", "..."):
                    vararg = True
                    break
                params.append(self.expect("name")[1])
                if not self.accept("op", ","):
                    break
        self.expect("op", ")")
        body = self.block()
        self.expect("kw", "end")
        return ("function", params, vararg, body, line)

    def explist(self):
        exps = [self.expr()]
        while self.accept("op", ","):
            exps.append(self.expr())
        return exps

    def primaryexp(self):
        tok = self.next()
        if tok[0] == "name":
            return ("name", tok[1], tok[2])
        if tok[0] == "op" and tok[1] == "(":
            e = self.expr()
            self.expect("op", ")")
            return ("paren", e)
        raise LuaError("line %d: unexpected %r" % (tok[2], tok[1]))

    def suffixedexp(self):
        e = self.primaryexp()
        while True:
            tok = self.peek()
            line = tok[2]
            if tok[0] == "op" and tok[1] == ".":
                self.next()
                e = ("index", e, ("const", self.expect("name")[1]), line)
            elif tok[0] == "op" and tok[1] == "[":
                self.next()
                k = self.expr()
                self.expect("op", "]")
                e = ("index", e, k, line)
            elif tok[0] == "op" and tok[1] == ":":
                self.next()
                name = self.expect("name")[1]
                e = ("method", e, name, self.callargs(), line)
            elif (tok[0] == "op" and tok[1] in ("(", "{")) or tok[0] == "str":
                e = ("call", e, self.callargs(), line)
            else:
                return e

    def callargs(self):
        tok = self.peek()
        if tok[0] == "str":
            self.next()
            return [("const", tok[1])]
        if tok[0] == "op" and tok[1] == "{":
            return [self.table()]
        self.expect("op", "(")
        if self.accept("op", ")"):
            return []
        args = self.explist()
        self.expect("op", ")")
        return args

    def table(self):
        self.expect("op", "{")
        items = []      # ("pos", e) | ("key", k, v)
        while not self.check("op", "}"):
            if self.check("op", "["):
                self.next()
                k = self.expr()
                self.expect("op", "]")
                self.expect("op", "=")
                items.append(("key", k, self.expr()))
            elif self.check("name") and self.peek(1)[0] == "op" and self.peek(1)[1] == "=":
                k = self.next()[1]
                self.next()
                items.append(("key", ("const", k), self.expr()))
            else:
                items.append(("pos", self.expr()))
            if not (self.accept("op", ",") or self.accept("op", ";")):
                break
        self.expect("op", "}")
        return ("table", items)

    def simpleexp(self):
        tok = self.peek()
        if tok[0] == "num":
            self.next()
            return ("const", tok[1])
        if tok[0] == "str":
            self.next()
            return ("const", tok[1])
        if tok[0] == "kw":
            if tok[1] == "nil":
                self.next()
                return ("const", None)
            if tok[1] == "true":
                self.next()
                return ("const", True)
            if tok[1] == "false":
                self.next()
                return ("const", False)
            if tok[1] == "function":
                self.next()
                return self.funcbody(False, tok[2])
        if tok[0] == "op":
            if tok[1] == "...":
                self.next()
                return ("vararg",)
            if tok[1] == "{":
                return self.table()
        return self.suffixedexp()

    def expr(self, limit=0):
        tok = self.peek()
        if (tok[0] == "kw" and tok[1] == "not") or (tok[0] == "op" and tok[1] in ("-", "#")):
            self.next()
            operand = self.expr(_UNARY_PRI)
            e = ("unop", tok[1], operand, tok[2])
        else:
            e = self.simpleexp()
        while True:
            tok = self.peek()
            op = tok[1] if tok[0] in ("op", "kw") else None
            if op not in _BINPRI or _BINPRI[op][0] <= limit:
                return e
            self.next()
            rhs = self.expr(_BINPRI[op][1])
            e = ("binop", op, e, rhs, tok[2])


# ---------------------------------------------------------------- runtime

class LuaTable:
    __slots__ = ("hash", "meta")

    def __init__(self):
        self.hash = {}
        self.meta = None

    def rawget(self, k):
        return self.hash.get(_key(k))

    def rawset(self, k, v):
        if k is None:
            raise LuaError("table index is nil")
        if isinstance(k, float) and k != k:
            raise LuaError("table index is NaN")
        kk = _key(k)
        if v is None:
            self.hash.pop(kk, None)
        else:
            self.hash[kk] = v

    def length(self):
        n = 0
        while (float(n + 1)) in self.hash:
            n += 1
        return n


class _BoolKey:
    """booleans as table keys (Python's True == 1.0 would collide)"""
    __slots__ = ("v",)

    def __init__(self, v):
        self.v = v

    def __hash__(self):
        return hash(("bool", self.v))

    def __eq__(self, o):
        return isinstance(o, _BoolKey) and o.v == self.v


def _key(k):
    if isinstance(k, bool):
        return _BoolKey(k)
    if isinstance(k, int):
        return float(k)
    return k


def _unkey(k):
    return k.v if isinstance(k, _BoolKey) else k


class LuaFunction:
    __slots__ = ("params", "vararg", "body", "scope", "interp", "name")

    def __init__(self, params, vararg, body, scope, interp, name="?"):
        self.params = params
        self.vararg = vararg
        self.body = body
        self.scope = scope
        self.interp = interp
        self.name = name


class _Break(Exception):
    pass


class _Return(Exception):
    def __init__(self, values):
        super().__init__()
        self.values = values


class Scope:
    __slots__ = ("vars", "parent", "varargs")

    def __init__(self, parent, varargs=None):
        self.vars = {}
        self.parent = parent
        self.varargs = varargs if varargs is not None else (parent.varargs if parent else [])

    def find(self, name):
        s = self
        while s is not None:
            if name in s.vars:
                return s
            s = s.parent
        return None


def lua_type(v):
    if v is None:
        return "nil"
    if isinstance(v, bool):
        return "boolean"
    if isinstance(v, (int, float)):
        return "number"
    if isinstance(v, str):
        return "string"
    if isinstance(v, LuaTable):
        return "table"
    if isinstance(v, LuaFunction) or callable(v):
        return "function"
    return "userdata"


def fmt_number(x):
    if isinstance(x, bool):
        raise LuaError("not a number")
    x = float(x)
    if x != x:
        return "nan" if math.copysign(1, x) > 0 else "-nan"
    if x == math.inf:
        return "inf"
    if x == -math.inf:
        return "-inf"
    return "%.14g" % x


def str2number(s):
    s = s.strip()
    try:
        if s[:2].lower() in ("0x",) or s[:3].lower() in ("-0x", "+0x"):
            return float(int(s, 16))
        if re.fullmatch(r"[+-]?(\d+\.?\d*|\.\d+)([eE][+-]?\d+)?", s):
            return float(s)
    except ValueError:
        return None
    return None


def truthy(v):
    return v is not None and v is not False


class Interp:
    def __init__(self, path=None, out=None):
        self.out = out or sys.stdout
        self.G = LuaTable()
        self.loaded = LuaTable()
        self.path = path or [os.getcwd()]
        self.string_lib = None
        self._install()

    # ---- helpers
    def getmeta(self, v):
        if isinstance(v, LuaTable):
            return v.meta
        if isinstance(v, str):
            return self.string_meta
        return None

    def metamethod(self, v, name):
        mt = self.getmeta(v)
        if mt is None:
            return None
        return mt.rawget(name)

    def tostring(self, v):
        mm = self.metamethod(v, "__tostring")
        if mm is not None:
            r = self.call(mm, [v])
            return r[0] if r else None
        if v is None:
            return "nil"
        if v is True:
            return "true"
        if v is False:
            return "false"
        if isinstance(v, (int, float)):
            return fmt_number(v)
        if isinstance(v, str):
            return v
        if isinstance(v, LuaTable):
            return "table: 0x%08x" % (id(v) & 0xffffffff)
        return "function: 0x%08x" % (id(v) & 0xffffffff)

    def tonum(self, v):
        if isinstance(v, bool):
            return None
        if isinstance(v, (int, float)):
            return float(v)
        if isinstance(v, str):
            return str2number(v)
        return None

    def index(self, obj, key):
        if isinstance(obj, LuaTable):
            v = obj.rawget(key)
            if v is not None:
                return v
            h = obj.meta.rawget("__index") if obj.meta is not None else None
            if h is None:
                return None
        else:
            h = self.metamethod(obj, "__index")
            if h is None:
                raise LuaError("attempt to index a %s value" % lua_type(obj))
        if isinstance(h, LuaTable) or isinstance(h, str):
            return self.index(h, key)
        r = self.call(h, [obj, key])
        return r[0] if r else None

    def setindex(self, obj, key, val):
        if isinstance(obj, LuaTable):
            if obj.meta is not None and obj.rawget(key) is None:
                h = obj.meta.rawget("__newindex")
                if h is not None:
                    if isinstance(h, LuaTable):
                        return self.setindex(h, key, val)
                    self.call(h, [obj, key, val])
                    return
            obj.rawset(key, val)
            return
        h = self.metamethod(obj, "__newindex")
        if h is None:
            raise LuaError("attempt to index a %s value" % lua_type(obj))
        if isinstance(h, LuaTable):
            return self.setindex(h, key, val)
        self.call(h, [obj, key, val])

    def call(self, f, args):
        if isinstance(f, LuaFunction):
            scope = Scope(f.scope, varargs=args[len(f.params):] if f.vararg else [])
            for i, p in enumerate(f.params):
                scope.vars[p] = args[i] if i < len(args) else None
            try:
                self.exec_block(f.body, scope)
            except _Return as r:
                return r.values
            return []
        if callable(f) and not isinstance(f, LuaTable):
            r = f(*args)
            if r is None:
                return []
            if isinstance(r, list):
                return r
            return [r]
        mm = self.metamethod(f, "__call")
        if mm is not None:
            return self.call(mm, [f] + list(args))
        raise LuaError("attempt to call a %s value" % lua_type(f))

    def arith(self, op, a, b):
        x, y = self.tonum(a), self.tonum(b)
        if x is not None and y is not None:
            if op == "+":
                return x + y
            if op == "-":
                return x - y
            if op == "*":
                return x*y
            if op == "/":
                if y == 0:
                    if x == 0 or x != x:
                        return math.nan
                    return math.copysign(math.inf, x)*math.copysign(1, y)
                return x/y
            if op == "%":
                if y == 0:
                    return math.nan
                return x - math.floor(x/y)*y
            if op == "^":
                return math.pow(x, y)
        ev = {"+": "__add", "-": "__sub", "*": "__mul", "/": "__div", "%": "__mod",
              "^": "__pow"}[op]
        mm = self.metamethod(a, ev)
        if mm is None:
            mm = self.metamethod(b, ev)
        if mm is None:
            bad = b if x is not None else a
            raise LuaError("attempt to perform arithmetic on a %s value" % lua_type(bad))
        r = self.call(mm, [a, b])
        return r[0] if r else None

    def concat(self, a, b):
        if isinstance(a, (str, int, float)) and not isinstance(a, bool) and \
           isinstance(b, (str, int, float)) and not isinstance(b, bool):
            sa = a if isinstance(a, str) else fmt_number(a)
            sb = b if isinstance(b, str) else fmt_number(b)
            return sa + sb
        mm = self.metamethod(a, "__concat") or self.metamethod(b, "__concat")
        if mm is None:
            bad = a if not isinstance(a, (str, int, float)) else b
            raise LuaError("attempt to concatenate a %s value" % lua_type(bad))
        r = self.call(mm, [a, b])
        return r[0] if r else None

    def equal(self, a, b):
        if lua_type(a) != lua_type(b):
            return False
        if isinstance(a, (int, float)) and not isinstance(a, bool):
            return float(a) == float(b)
        if a is b or (isinstance(a, str) and a == b) or (isinstance(a, bool) and a == b):
            return True
        if isinstance(a, LuaTable) and isinstance(b, LuaTable):
            m1 = self.metamethod(a, "__eq")
            m2 = self.metamethod(b, "__eq")
            if m1 is not None and m1 is m2:
                r = self.call(m1, [a, b])
                return truthy(r[0] if r else None)
        return False

    def less(self, a, b, ev="__lt"):
        if isinstance(a, (int, float)) and isinstance(b, (int, float)) and \
           not isinstance(a, bool) and not isinstance(b, bool):
            return a < b if ev == "__lt" else a <= b
        if isinstance(a, str) and isinstance(b, str):
            return a < b if ev == "__lt" else a <= b
        m1 = self.metamethod(a, ev)
        m2 = self.metamethod(b, ev)
        if m1 is not None and m1 is m2:
            r = self.call(m1, [a, b])
            return truthy(r[0] if r else None)
        if ev == "__le":
            m1 = self.metamethod(a, "__lt")
            m2 = self.metamethod(b, "__lt")
            if m1 is not None and m1 is m2:
                r = self.call(m1, [b, a])
                return not truthy(r[0] if r else None)
        raise LuaError("attempt to compare %s with %s" % (lua_type(a), lua_type(b)))

    # ---- evaluation
    def eval_multi(self, exps, scope):
        """values of an expression list: the last call or ... expands"""
        vals = []
        for i, e in enumerate(exps):
            if i == len(exps) - 1 and e[0] in ("call", "method", "vararg"):
                vals.extend(self.eval_m(e, scope))
            else:
                vals.append(self.eval(e, scope))
        return vals

    def eval_m(self, e, scope):
        k = e[0]
        if k == "vararg":
            return list(scope.varargs)
        if k == "call":
            f = self.eval(e[1], scope)
            args = self.eval_multi(e[2], scope)
            try:
                return self.call(f, args)
            except LuaError as err:
                if not err.where:
                    err.where = "line %d" % e[3]
                raise
        if k == "method":
            obj = self.eval(e[1], scope)
            f = self.index(obj, e[2])
            args = [obj] + self.eval_multi(e[3], scope)
            try:
                return self.call(f, args)
            except LuaError as err:
                if not err.where:
                    err.where = "line %d" % e[4]
                raise
        return [self.eval(e, scope)]

    def eval(self, e, scope):
        k = e[0]
        if k == "const":
            return e[1]
        if k == "name":
            s = scope.find(e[1])
            if s is not None:
                return s.vars[e[1]]
            return self.G.rawget(e[1])
        if k == "index":
            obj = self.eval(e[1], scope)
            key = self.eval(e[2], scope)
            try:
                return self.index(obj, key)
            except LuaError as err:
                if not err.where:
                    err.where = "line %d" % e[3]
                raise
        if k in ("call", "method", "vararg"):
            r = self.eval_m(e, scope)
            return r[0] if r else None
        if k == "paren":
            return self.eval(e[1], scope)
        if k == "binop":
            op = e[1]
            if op == "and":
                a = self.eval(e[2], scope)
                return self.eval(e[3], scope) if truthy(a) else a
            if op == "or":
                a = self.eval(e[2], scope)
                return a if truthy(a) else self.eval(e[3], scope)
            a = self.eval(e[2], scope)
            b = self.eval(e[3], scope)
            try:
                if op in ("+", "-", "*", "/", "%", "^"):
                    return self.arith(op, a, b)
                if op == "..":
                    return self.concat(a, b)
                if op == "==":
                    return self.equal(a, b)
                if op == "~=":
                    return not self.equal(a, b)
                if op == "<":
                    return self.less(a, b)
                if op == "<=":
                    return self.less(a, b, "__le")
                if op == ">":
                    return self.less(b, a)
                if op == ">=":
                    return self.less(b, a, "__le")
            except LuaError as err:
                if not err.where:
                    err.where = "line %d" % e[4]
                raise
            raise LuaError("unknown operator " + op)
        if k == "unop":
            op = e[1]
            v = self.eval(e[2], scope)
            if op == "not":
                return not truthy(v)
            if op == "-":
                x = self.tonum(v)
                if x is not None:
                    return -x
                mm = self.metamethod(v, "__unm")
                if mm is None:
                    raise LuaError("attempt to perform arithmetic on a %s value" % lua_type(v),
                                   "line %d" % e[3])
                r = self.call(mm, [v, v])
                return r[0] if r else None
            if op == "#":
                if isinstance(v, str):
                    return float(len(v))
                mm = self.metamethod(v, "__len")
                if mm is not None and not isinstance(v, LuaTable):
                    r = self.call(mm, [v])
                    return r[0] if r else None
                if isinstance(v, LuaTable):
                    return float(v.length())
                raise LuaError("attempt to get length of a %s value" % lua_type(v),
                               "line %d" % e[3])
        if k == "function":
            return LuaFunction(e[1], e[2], e[3], scope, self, "line %d" % e[4])
        if k == "table":
            t = LuaTable()
            n = 1
            items = e[1]
            for i, it in enumerate(items):
                if it[0] == "key":
                    t.rawset(self.eval(it[1], scope), self.eval(it[2], scope))
                elif i == len(items) - 1 and it[1][0] in ("call", "method", "vararg"):
                    for v in self.eval_m(it[1], scope):
                        t.rawset(float(n), v)
                        n += 1
                else:
                    t.rawset(float(n), self.eval(it[1], scope))
                    n += 1
            return t
        raise LuaError("cannot evaluate " + k)

    def assign(self, target, val, scope):
        if target[0] == "name":
            s = scope.find(target[1])
            if s is not None:
                s.vars[target[1]] = val
            else:
                self.G.rawset(target[1], val)
        else:
            obj = self.eval(target[1], scope)
            key = self.eval(target[2], scope)
            try:
                self.setindex(obj, key, val)
            except LuaError as err:
                if not err.where:
                    err.where = "line %d" % target[3]
                raise

    def exec_block(self, stats, scope):
        for st in stats:
            self.exec(st, scope)

    def exec(self, st, scope):
        k = st[0]
        if k == "exprstat":
            self.eval_m(st[1], scope)
        elif k == "local":
            vals = self.eval_multi(st[2], scope)
            for i, name in enumerate(st[1]):
                scope.vars[name] = vals[i] if i < len(vals) else None
        elif k == "assign":
            targets, exps = st[1], st[2]
            # evaluate the right-hand side first, then assign
            vals = self.eval_multi(exps, scope)
            for i, t in enumerate(targets):
                self.assign(t, vals[i] if i < len(vals) else None, scope)
        elif k == "localfunc":
            scope.vars[st[1]] = None
            scope.vars[st[1]] = self.eval(st[2], scope)
        elif k == "if":
            for cond, body in st[1]:
                if truthy(self.eval(cond, scope)):
                    self.exec_block(body, Scope(scope))
                    return
            if st[2] is not None:
                self.exec_block(st[2], Scope(scope))
        elif k == "fornum":
            name, a, b, c, body, line = st[1:]
            start = self.tonum(self.eval(a, scope))
            stop = self.tonum(self.eval(b, scope))
            step = self.tonum(self.eval(c, scope)) if c is not None else 1.0
            if start is None or stop is None or step is None:
                raise LuaError("'for' initial value, limit and step must be numbers", "line %d" % line)
            v = start
            try:
                while (step > 0 and v <= stop) or (step <= 0 and v >= stop):
                    inner = Scope(scope)
                    inner.vars[name] = v
                    self.exec_block(body, inner)
                    v += step
            except _Break:
                pass
        elif k == "forin":
            names, exps, body, line = st[1:]
            vals = self.eval_multi(exps, scope)
            f = vals[0] if vals else None
            s = vals[1] if len(vals) > 1 else None
            var = vals[2] if len(vals) > 2 else None
            try:
                while True:
                    r = self.call(f, [s, var])
                    if not r or r[0] is None:
                        break
                    var = r[0]
                    inner = Scope(scope)
                    for i, nm in enumerate(names):
                        inner.vars[nm] = r[i] if i < len(r) else None
                    self.exec_block(body, inner)
            except _Break:
                pass
        elif k == "while":
            try:
                while truthy(self.eval(st[1], scope)):
                    self.exec_block(st[2], Scope(scope))
            except _Break:
                pass
        elif k == "repeat":
            try:
                while True:
                    inner = Scope(scope)
                    self.exec_block(st[1], inner)
                    # the condition sees the body's locals
                    if truthy(self.eval(st[2], inner)):
                        break
            except _Break:
                pass
        elif k == "do":
            self.exec_block(st[1], Scope(scope))
        elif k == "return":
            raise _Return(self.eval_multi(st[1], scope))
        elif k == "break":
            raise _Break()
        else:
            raise LuaError("unknown statement " + k)

    # ---- library
    def _install(self):
        G = self.G
        I = self

        def setf(t, name, f):
            t.rawset(name, f)

        def lua_print(*args):
            I.out.write("\t".join(I.tostring(a) for a in args) + "\n")

        def lua_tostring(v=None, *_):
            return I.tostring(v)

        def lua_tonumber(v=None, base=None, *_):
            if base is None:
                return I.tonum(v)
            try:
                return float(int(str(v).strip(), int(base)))
            except ValueError:
                return None

        def lua_setmetatable(t, mt=None, *_):
            if not isinstance(t, LuaTable):
                raise LuaError("bad argument #1 to 'setmetatable' (table expected)")
            t.meta = mt
            return t

        def lua_getmetatable(v=None, *_):
            mt = I.getmeta(v)
            if mt is None:
                return None
            prot = mt.rawget("__metatable")
            return prot if prot is not None else mt

        def lua_type_(v=None, *_):
            return lua_type(v)

        def lua_next(t, k=None, *_):
            keys = list(t.hash.keys())
            if k is None:
                idx = 0
            else:
                try:
                    idx = keys.index(_key(k)) + 1
                except ValueError:
                    raise LuaError("invalid key to 'next'")
            if idx >= len(keys):
                return [None]
            kk = keys[idx]
            return [_unkey(kk), t.hash[kk]]

        def lua_pairs(t, *_):
            mm = I.metamethod(t, "__pairs")
            if mm is not None:
                return I.call(mm, [t])[:3]
            return [lua_next, t, None]

        def ipairs_iter(t, i):
            i = i + 1
            v = I.index(t, i)
            if v is None:
                return [None]
            return [i, v]

        def lua_ipairs(t, *_):
            return [ipairs_iter, t, 0.0]

        def lua_select(n, *args):
            if n == "#":
                return float(len(args))
            n = int(n)
            if n < 0:
                n = len(args) + n + 1
            return list(args[n - 1:])

        def lua_unpack(t, i=1.0, j=None, *_):
            i = int(i)
            j = t.length() if j is None else int(j)
            return [t.rawget(float(k)) for k in range(i, j + 1)]

        def lua_assert(v=None, msg=None, *rest):
            if not truthy(v):
                raise LuaError(msg if msg is not None else "assertion failed!")
            return [v, msg] + list(rest)

        def lua_error(msg=None, *_):
            raise LuaError(msg)

        def lua_pcall(f, *args):
            try:
                return [True] + I.call(f, list(args))
            except LuaError as err:
                return [False, err.value]

        def lua_rawget(t, k, *_):
            return t.rawget(k)

        def lua_rawset(t, k, v, *_):
            t.rawset(k, v)
            return t

        def lua_rawequal(a, b, *_):
            return a is b or (lua_type(a) == lua_type(b) and lua_type(a) in ("number", "string",
                                                                               "boolean")
                              and a == b)

        def lua_require(name, *_):
            v = I.loaded.rawget(name)
            if v is not None:
                return v
            for d in I.path:
                p = os.path.join(d, name.replace(".", os.sep) + ".lua")
                if os.path.exists(p):
                    r = I.run_file(p)
                    val = r[0] if r and r[0] is not None else True
                    if I.loaded.rawget(name) is None:
                        I.loaded.rawset(name, val)
                    return I.loaded.rawget(name)
            raise LuaError("module '%s' not found" % name)

        for name, f in (("print", lua_print), ("tostring", lua_tostring),
                        ("tonumber", lua_tonumber), ("setmetatable", lua_setmetatable),
                        ("getmetatable", lua_getmetatable), ("type", lua_type_),
                        ("next", lua_next), ("pairs", lua_pairs), ("ipairs", lua_ipairs),
                        ("select", lua_select), ("unpack", lua_unpack), ("assert", lua_assert),
                        ("error", lua_error), ("pcall", lua_pcall), ("rawget", lua_rawget),
                        ("rawset", lua_rawset), ("rawequal", lua_rawequal),
                        ("require", lua_require)):
            setf(G, name, f)
        G.rawset("_G", G)
        G.rawset("_VERSION", "Lua 5.1")

        # string
        S = LuaTable()

        def s_format(fmt, *args):
            return I.format(fmt, args)

        def s_rep(s, n, *_):
            n = int(n)
            return I.tostring(s)*max(n, 0)

        def s_sub(s, i=1.0, j=-1.0, *_):
            s = I.tostring(s) if not isinstance(s, str) else s
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
            return s[i - 1:j] if i <= j else ""

        def s_len(s, *_):
            return float(len(s))

        def s_upper(s, *_):
            return s.upper()

        def s_lower(s, *_):
            return s.lower()

        def s_byte(s, i=1.0, j=None, *_):
            i = int(i)
            j = i if j is None else int(j)
            return [float(ord(c)) for c in s[i - 1:j]]

        def s_char(*args):
            return "".join(chr(int(a)) for a in args)

        for name, f in (("format", s_format), ("rep", s_rep), ("sub", s_sub), ("len", s_len),
                        ("upper", s_upper), ("lower", s_lower), ("byte", s_byte),
                        ("char", s_char)):
            setf(S, name, f)
        G.rawset("string", S)
        self.string_meta = LuaTable()
        self.string_meta.rawset("__index", S)

        # table
        T = LuaTable()

        def t_insert(t, *args):
            if len(args) == 1:
                t.rawset(float(t.length() + 1), args[0])
            else:
                pos, v = int(args[0]), args[1]
                n = t.length()
                for k in range(n, pos - 1, -1):
                    t.rawset(float(k + 1), t.rawget(float(k)))
                t.rawset(float(pos), v)

        def t_remove(t, pos=None, *_):
            n = t.length()
            if n == 0:
                return None
            pos = n if pos is None else int(pos)
            v = t.rawget(float(pos))
            for k in range(pos, n):
                t.rawset(float(k), t.rawget(float(k + 1)))
            t.rawset(float(n), None)
            return v

        def t_concat(t, sep="", i=1.0, j=None, *_):
            j = t.length() if j is None else int(j)
            return sep.join(I.tostring(t.rawget(float(k))) for k in range(int(i), j + 1))

        for name, f in (("insert", t_insert), ("remove", t_remove), ("concat", t_concat)):
            setf(T, name, f)
        G.rawset("table", T)

        # math
        M = LuaTable()
        for name, f in (("floor", lambda x, *_: float(math.floor(x))),
                        ("ceil", lambda x, *_: float(math.ceil(x))),
                        ("abs", lambda x, *_: abs(float(x))),
                        ("sqrt", lambda x, *_: math.sqrt(x)),
                        ("max", lambda *a: float(max(a))), ("min", lambda *a: float(min(a))),
                        ("sin", lambda x, *_: math.sin(x)), ("cos", lambda x, *_: math.cos(x)),
                        ("exp", lambda x, *_: math.exp(x)), ("log", lambda x, *_: math.log(x)),
                        ("fmod", lambda a, b, *_: math.fmod(a, b))):
            setf(M, name, f)
        M.rawset("pi", math.pi)
        M.rawset("huge", math.inf)
        G.rawset("math", M)

        # io
        IO = LuaTable()

        def io_write(*args):
            for a in args:
                I.out.write(a if isinstance(a, str) else fmt_number(a))

        setf(IO, "write", io_write)
        G.rawset("io", IO)

    _SPEC = re.compile(r"%([-+ #0]*)(\d*)(?:\.(\d*))?([diouxXeEfgGcqs%])")

    def format(self, fmt, args):
        out = []
        pos = 0
        ai = 0
        for m in self._SPEC.finditer(fmt):
            out.append(fmt[pos:m.start()])
            pos = m.end()
            flags, width, prec, conv = m.group(1), m.group(2), m.group(3), m.group(4)
            if conv == "%":
                out.append("%")
                continue
            if ai >= len(args):
                raise LuaError("bad argument #%d to 'format' (no value)" % (ai + 2))
            a = args[ai]
            ai += 1
            spec = "%" + flags + width + ("." + prec if prec is not None else "")
            if conv in "di":
                x = self.tonum(a)
                if x is None:
                    raise LuaError("bad argument #%d to 'format' (number expected)" % (ai + 1))
                out.append((spec + "d") % int(x))
            elif conv in "ouxX":
                x = self.tonum(a)
                if x is None:
                    raise LuaError("bad argument #%d to 'format' (number expected)" % (ai + 1))
                out.append((spec + conv) % int(x))
            elif conv in "eEfgG":
                x = self.tonum(a)
                if x is None:
                    raise LuaError("bad argument #%d to 'format' (number expected)" % (ai + 1))
                out.append((spec + conv) % x)
            elif conv == "c":
                out.append(chr(int(self.tonum(a))))
            elif conv == "q":
                s = self.tostring(a)
                out.append('"' + s.replace("\\", "\\\\").replace('"', '\\"')
                           .replace("\n", "\\\n").replace("\r", "\\r").replace("\0", "\\000")
                           + '"')
            else:  # s
                s = self.tostring(a)
                out.append((spec + "s") % s)
        out.append(fmt[pos:])
        return "".join(out)

    # ---- entry points
    def run_source(self, src, name="?"):
        ast = Parser(tokenize(src)).block()
        scope = Scope(None, varargs=[])
        try:
            self.exec_block(ast, scope)
        except _Return as r:
            return r.values
        except LuaError as err:
            raise LuaError("%s:%s: %s" % (name, err.where, err.value)) from None
        return []

    def run_file(self, path):
        with open(path) as f:
            return self.run_source(f.read(), os.path.basename(path))


def run_script(path, out):
    """runs a Lua script as `lua path > out` would from its own directory"""
    d = os.path.dirname(os.path.abspath(path))
    interp = Interp(path=[d], out=out)
    interp.run_file(path)


if __name__ == "__main__":
    run_script(sys.argv[1], sys.stdout)
