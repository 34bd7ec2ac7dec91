"""A small interpreter for the subset of MATLAB that BristolFE-v2's hot-path
files use - test infrastructure only.

No MATLAB or GNU Octave exists on this machine, so this module runs the
reference's own ``.m`` files (unmodified, read from a reference checkout) to
produce golden vectors: mesh generation, global assembly, element routines,
the v6 and v5 explicit solvers, field output and the ``fn_BristolFE_v2``
entry point. It parses MATLAB source into a syntax tree and evaluates it
with MATLAB's semantics (column-major arrays of at least two dimensions,
1-based indexing with growth and deletion, implicit expansion, logical
indexing, structs and struct arrays, cell arrays, comma-separated lists,
sparse matrices, ``end`` in subscripts, varargin/varargout/nargin/nargout).
MATLAB's built-in functions that those files call are restated here on
NumPy/SciPy from their documented behaviour (``sparse`` sums duplicates,
``unique`` sorts, ``interp1(..., 'nearest')``, ``inpolygon`` counts points
on the boundary as inside, ...). Only arithmetic is offered: there is no
file, system or graphics access, and an unknown function is an error.
"""
import math
import os
import re

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla


class MatlabError(Exception):
    """An error() raised by the interpreted code, or an unsupported construct."""


# ---------------------------------------------------------------------------
# values

class Char(str):
    """A MATLAB char row vector."""

    @property
    def mshape(self):
        return (1, len(self)) if len(self) else (0, 0)


class Cell:
    """A MATLAB cell array: an object ndarray of at least two dimensions."""

    def __init__(self, arr):
        arr = np.asarray(arr, dtype=object) if not isinstance(arr, np.ndarray) else arr
        if arr.ndim < 2:
            arr = arr.reshape((1, -1) if arr.size else (0, 0))
        self.a = arr

    @staticmethod
    def empty(shape=(0, 0)):
        a = np.empty(shape, dtype=object)
        for k in np.ndindex(a.shape):
            a[k] = empty_double()
        return Cell(a)


class Struct:
    """A MATLAB struct array: an object ndarray of dicts plus the field order."""

    def __init__(self, arr=None, fields=None):
        if arr is None:
            arr = np.empty((1, 1), dtype=object)
            arr[0, 0] = {}
        self.a = arr
        self.fields = list(fields or [])
        for d in self.a.flat:
            for k in d:
                if k not in self.fields:
                    self.fields.append(k)

    def copy(self):
        b = np.empty(self.a.shape, dtype=object)
        for k in np.ndindex(self.a.shape):
            b[k] = dict(self.a[k])
        return Struct(b, self.fields)


class Handle:
    """A function handle (by name)."""

    def __init__(self, name):
        self.name = name


class CSL(list):
    """A comma-separated list (struct array field, cell brace indexing)."""


def empty_double():
    return np.zeros((0, 0))


def to_m(v):
    """Python/NumPy value -> MATLAB value."""
    if isinstance(v, (Char, Cell, Struct, Handle)) or sp.issparse(v):
        return v
    if isinstance(v, str):
        return Char(v)
    if isinstance(v, dict):
        s = Struct()
        for k, x in v.items():
            s.a[0, 0][k] = to_m(x)
            s.fields.append(k)
        return s
    if isinstance(v, (list, tuple)) and v and all(isinstance(x, dict) for x in v):
        arr = np.empty((len(v), 1), dtype=object)
        fields = []
        for i, d in enumerate(v):
            arr[i, 0] = {k: to_m(x) for k, x in d.items()}
            for k in d:
                if k not in fields:
                    fields.append(k)
        return Struct(arr, fields)
    if isinstance(v, (list, tuple)) and v and any(isinstance(x, str) for x in v):
        arr = np.empty((len(v), 1), dtype=object)
        for i, x in enumerate(v):
            arr[i, 0] = to_m(x)
        return Cell(arr)
    a = np.asarray(v)
    if a.dtype.kind in "iu":
        a = a.astype(np.float64)
    if a.ndim == 0:
        a = a.reshape(1, 1)
    elif a.ndim == 1:
        a = a.reshape(1, -1)
    return a


# ---------------------------------------------------------------------------
# lexer

KEYWORDS = {"function", "end", "if", "elseif", "else", "for", "while", "switch", "case", "otherwise",
            "break", "continue", "return", "try", "catch", "global", "persistent", "parfor"}
_OPS = ["...", ".^", ".*", "./", ".\\", ".'", "==", "~=", "<=", ">=", "&&", "||", "!=",
        "+", "-", "*", "/", "\\", "^", "<", ">", "&", "|", "~", "!", "=", "(", ")", "[", "]",
        "{", "}", ",", ";", ":", ".", "@", "'", "\n"]


class Tok:
    __slots__ = ("kind", "val", "line")

    def __init__(self, kind, val, line):
        self.kind, self.val, self.line = kind, val, line

    def __repr__(self):
        return "Tok(%s,%r)" % (self.kind, self.val)


def _value_end(t):
    return t is not None and (t.kind in ("num", "str", "id") or
                              (t.kind == "op" and t.val in (")", "]", "}", "'", ".'")) or
                              (t.kind == "kw" and t.val == "end"))


def lex(src):
    """Tokens of MATLAB source; whitespace that separates elements inside
    [] and {} becomes ',' and newlines there become ';'."""
    toks = []
    i, n, line = 0, len(src), 1
    stack = []                     # bracket kinds: '(', '[', '{'
    prev = None
    in_block_comment = False
    while i < n:
        c = src[i]
        # block comments: lines holding only %{ ... %}
        if c in " \t" or (c == "%" and not in_block_comment):
            pass
        if in_block_comment:
            j = src.find("\n", i)
            j = n if j < 0 else j
            if src[i:j].strip() == "%}":
                in_block_comment = False
            i = j + 1 if j < n else n
            line += 1
            continue
        if c == "%":
            j = src.find("\n", i)
            j = n if j < 0 else j
            lstart = src.rfind("\n", 0, i) + 1
            if src[i:j].strip() == "%{" and src[lstart:i].strip() == "":
                in_block_comment = True
                i = j + 1
                line += 1
                continue
            i = j
            continue
        if src.startswith("...", i):
            j = src.find("\n", i)
            i = n if j < 0 else j + 1
            line += 1
            continue
        in_mat = bool(stack) and stack[-1] in "[{"
        if c in " \t\r":
            j = i
            while j < n and src[j] in " \t\r":
                j += 1
            if in_mat and _value_end(prev) and j < n:
                d = src[j]
                nxt2 = src[j + 1] if j + 1 < n else ""
                starts_value = (d.isalnum() or d in "_([{'\"@" or (d == "." and nxt2.isdigit()) or
                                (d in "~!" and nxt2 != "=") or
                                (d in "+-" and nxt2 not in " \t=" and not src.startswith("...", j)))
                if starts_value and not src.startswith("...", j):
                    toks.append(Tok("op", ",", line))
                    prev = toks[-1]
            i = j
            continue
        if c == "\n":
            if in_mat:
                if prev is not None and not (prev.kind == "op" and prev.val in (";", ",", "[", "{")):
                    toks.append(Tok("op", ";", line))
                    prev = toks[-1]
            elif not stack:
                toks.append(Tok("op", "\n", line))
                prev = toks[-1]
            line += 1
            i += 1
            continue
        if c.isdigit() or (c == "." and i + 1 < n and src[i + 1].isdigit()):
            m = re.match(r"(\d+\.?\d*|\.\d+)([eE][+-]?\d+)?", src[i:])
            toks.append(Tok("num", float(m.group(0)), line))
            prev = toks[-1]
            i += len(m.group(0))
            continue
        if c.isalpha() or c == "_":
            m = re.match(r"[A-Za-z_]\w*", src[i:])
            w = m.group(0)
            kind = "kw" if w in KEYWORDS else "id"
            # 'end' inside () or {} subscripts is a value
            if w == "end" and stack and stack[-1] in "({":
                kind = "kw"
            toks.append(Tok(kind, w, line))
            prev = toks[-1]
            i += len(w)
            continue
        if c == "'" and _value_end(prev) and i > 0 and src[i - 1] not in " \t":
            toks.append(Tok("op", "'", line))
            prev = toks[-1]
            i += 1
            continue
        if c == "'" and not (_value_end(prev) and not in_mat):
            j = i + 1
            buf = []
            while True:
                if j >= n or src[j] == "\n":
                    raise MatlabError("unterminated string on line %d" % line)
                if src[j] == "'":
                    if j + 1 < n and src[j + 1] == "'":
                        buf.append("'")
                        j += 2
                        continue
                    break
                buf.append(src[j])
                j += 1
            toks.append(Tok("str", "".join(buf), line))
            prev = toks[-1]
            i = j + 1
            continue
        if c == '"':
            j = i + 1
            buf = []
            while src[j] != '"' or (j + 1 < n and src[j + 1] == '"'):
                if src[j] == '"':
                    j += 1
                buf.append(src[j])
                j += 1
            toks.append(Tok("str", "".join(buf), line))
            prev = toks[-1]
            i = j + 1
            continue
        for op in _OPS:
            if src.startswith(op, i):
                break
        else:
            raise MatlabError("unexpected character %r on line %d" % (c, line))
        if op in ("(", "[", "{"):
            stack.append(op)
        elif op in (")", "]", "}"):
            if stack:
                stack.pop()
        if op == "!=":
            op = "~="
        if op == "!":
            op = "~"
        toks.append(Tok("op", op, line))
        prev = toks[-1]
        i += len(op)
    toks.append(Tok("op", "\n", line))
    toks.append(Tok("eof", None, line))
    return toks


# ---------------------------------------------------------------------------
# parser: statements and expressions as tuples

class Parser:
    def __init__(self, toks):
        self.t = toks
        self.i = 0

    def peek(self, k=0):
        return self.t[self.i + k]

    def at(self, kind, val=None):
        tk = self.t[self.i]
        return tk.kind == kind and (val is None or tk.val == val)

    def at_op(self, *vals):
        tk = self.t[self.i]
        return tk.kind == "op" and tk.val in vals

    def at_kw(self, *vals):
        tk = self.t[self.i]
        return tk.kind == "kw" and tk.val in vals

    def next(self):
        tk = self.t[self.i]
        self.i += 1
        return tk

    def expect_op(self, v):
        tk = self.next()
        if tk.kind != "op" or tk.val != v:
            raise MatlabError("expected %r, got %r on line %d" % (v, tk.val, tk.line))
        return tk

    def skip_newlines(self):
        while self.at_op("\n", ";", ","):
            self.i += 1

    # -- file ------------------------------------------------------------
    def parse_file(self):
        funcs = {}
        order = []
        self.skip_newlines()
        if not self.at_kw("function"):
            body = self.block(("eof",))
            return {"__script__": ("function", "__script__", [], [], body)}, ["__script__"]
        while not self.at("eof"):
            f = self.function()
            funcs[f[1]] = f
            order.append(f[1])
            self.skip_newlines()
        return funcs, order

    def function(self):
        self.next()                                         # 'function'
        outs = []
        # [a, b] = name(...), a = name(...), name(...)
        save = self.i
        if self.at_op("["):
            self.next()
            while not self.at_op("]"):
                if self.at_op(","):
                    self.next()
                    continue
                outs.append(self.next().val)
            self.next()
            self.expect_op("=")
        else:
            tk = self.next()
            if self.at_op("="):
                self.next()
                outs = [tk.val]
            else:
                self.i = save
        name = self.next().val
        while self.at_op("."):                               # (no dotted names in these files)
            self.next()
            name += "." + self.next().val
        params = []
        if self.at_op("("):
            self.next()
            while not self.at_op(")"):
                if self.at_op(","):
                    self.next()
                    continue
                tk = self.next()
                params.append("~" if (tk.kind == "op" and tk.val == "~") else tk.val)
            self.next()
        body = self.block(("end", "function", "eof"))
        if self.at_kw("end"):
            self.next()
        return ("function", name, params, outs, body)

    def block(self, terms):
        out = []
        while True:
            self.skip_newlines()
            tk = self.peek()
            if tk.kind == "eof" and "eof" in terms:
                return out
            if tk.kind == "kw" and tk.val in terms:
                return out
            if tk.kind == "eof":
                raise MatlabError("unexpected end of file")
            out.append(self.statement())

    def end_stmt(self):
        tk = self.peek()
        if tk.kind == "op" and tk.val in ("\n", ";", ","):
            self.next()
        elif tk.kind != "eof" and not (tk.kind == "kw" and tk.val in ("end", "else", "elseif", "case",
                                                                       "otherwise", "catch", "function")):
            raise MatlabError("unexpected %r on line %d" % (tk.val, tk.line))

    def statement(self):
        tk = self.peek()
        line = tk.line
        if tk.kind == "kw":
            v = tk.val
            if v == "if":
                self.next()
                clauses = []
                cond = self.expr()
                body = self.block(("elseif", "else", "end"))
                clauses.append((cond, body))
                els = []
                while True:
                    if self.at_kw("elseif"):
                        self.next()
                        cond = self.expr()
                        body = self.block(("elseif", "else", "end"))
                        clauses.append((cond, body))
                    elif self.at_kw("else"):
                        self.next()
                        els = self.block(("end",))
                    else:
                        break
                self.next()
                return ("if", clauses, els, line)
            if v in ("for", "parfor"):
                self.next()
                paren = self.at_op("(")
                if paren:
                    self.next()
                var = self.next().val
                self.expect_op("=")
                rng = self.expr()
                if paren:
                    self.expect_op(")")
                body = self.block(("end",))
                self.next()
                return ("for", var, rng, body, line)
            if v == "while":
                self.next()
                cond = self.expr()
                body = self.block(("end",))
                self.next()
                return ("while", cond, body, line)
            if v == "switch":
                self.next()
                e = self.expr()
                cases = []
                other = None
                self.skip_newlines()
                while True:
                    self.skip_newlines()
                    if self.at_kw("case"):
                        self.next()
                        ce = self.expr()
                        body = self.block(("case", "otherwise", "end"))
                        cases.append((ce, body))
                    elif self.at_kw("otherwise"):
                        self.next()
                        other = self.block(("case", "otherwise", "end"))
                    else:
                        break
                self.next()
                return ("switch", e, cases, other or [], line)
            if v == "try":
                self.next()
                body = self.block(("catch", "end"))
                var, cbody = None, []
                if self.at_kw("catch"):
                    self.next()
                    if self.at("id") and self.peek(1).kind == "op" and self.peek(1).val == "\n":
                        var = self.next().val
                    cbody = self.block(("end",))
                self.next()
                return ("try", body, var, cbody, line)
            if v in ("break", "continue", "return"):
                self.next()
                self.end_stmt()
                return (v, line)
            if v in ("global", "persistent"):
                self.next()
                names = []
                while self.at("id"):
                    names.append(self.next().val)
                self.end_stmt()
                return ("global", names, line)
            raise MatlabError("unexpected keyword %r on line %d" % (v, line))
        # multiple assignment [a, b] = ...
        if tk.kind == "op" and tk.val == "[":
            j = self._match(self.i)
            if j is not None and self.t[j + 1].kind == "op" and self.t[j + 1].val == "=" and \
                    not (self.t[j + 2].kind == "op" and self.t[j + 2].val == "="):
                self.next()
                lhs = []
                while not self.at_op("]"):
                    if self.at_op(","):
                        self.next()
                        continue
                    if self.at_op("~"):
                        self.next()
                        lhs.append(None)
                        continue
                    lhs.append(self.postfix_expr())
                self.next()
                self.expect_op("=")
                rhs = self.expr()
                printed = not self.at_op(";")
                self.end_stmt()
                return ("assign", lhs, rhs, printed, line)
        # command syntax is not used by these files
        e = self.expr()
        if self.at_op("="):
            self.next()
            rhs = self.expr()
            printed = not self.at_op(";")
            self.end_stmt()
            return ("assign", [e], rhs, printed, line)
        printed = not self.at_op(";")
        self.end_stmt()
        return ("expr", e, printed, line)

    def _match(self, i):
        depth = 0
        for j in range(i, len(self.t)):
            tk = self.t[j]
            if tk.kind == "op" and tk.val in ("[", "(", "{"):
                depth += 1
            elif tk.kind == "op" and tk.val in ("]", ")", "}"):
                depth -= 1
                if depth == 0:
                    return j
            elif tk.kind == "op" and tk.val == "\n" and depth == 0:
                return None
        return None

    # -- expressions (MATLAB precedence, lowest first) ---------------------
    def expr(self):
        return self.oror()

    def oror(self):
        a = self.andand()
        while self.at_op("||"):
            self.next()
            a = ("oror", a, self.andand())
        return a

    def andand(self):
        a = self.elor()
        while self.at_op("&&"):
            self.next()
            a = ("andand", a, self.elor())
        return a

    def elor(self):
        a = self.eland()
        while self.at_op("|"):
            self.next()
            a = ("bin", "|", a, self.eland())
        return a

    def eland(self):
        a = self.cmp()
        while self.at_op("&"):
            self.next()
            a = ("bin", "&", a, self.cmp())
        return a

    def cmp(self):
        a = self.rng()
        while self.at_op("==", "~=", "<", "<=", ">", ">="):
            op = self.next().val
            a = ("bin", op, a, self.rng())
        return a

    def rng(self):
        if self.at_op(":") and self._bare_colon():
            self.next()
            return ("colon_all",)
        a = self.add()
        if self.at_op(":"):
            self.next()
            b = self.add()
            if self.at_op(":"):
                self.next()
                c = self.add()
                return ("range", a, b, c)
            return ("range", a, None, b)
        return a

    def _bare_colon(self):
        nx = self.peek(1)
        return nx.kind == "op" and nx.val in (",", ")", "}")

    def add(self):
        a = self.mul()
        while self.at_op("+", "-"):
            op = self.next().val
            a = ("bin", op, a, self.mul())
        return a

    def mul(self):
        a = self.unary()
        while self.at_op("*", "/", "\\", ".*", "./", ".\\"):
            op = self.next().val
            a = ("bin", op, a, self.unary())
        return a

    def unary(self):
        if self.at_op("-", "+", "~"):
            op = self.next().val
            return ("un", op, self.unary())
        return self.power()

    def power(self):
        a = self.postfix_expr()
        while self.at_op("^", ".^"):
            op = self.next().val
            if self.at_op("-", "+", "~"):                 # 2^-1
                uop = self.next().val
                b = ("un", uop, self.postfix_expr())
            else:
                b = self.postfix_expr()
            a = ("bin", op, a, b)
        return a

    def postfix_expr(self):
        a = self.primary()
        while True:
            if self.at_op("("):
                self.next()
                args = self.args(")")
                a = ("index", a, args)
            elif self.at_op("{"):
                self.next()
                args = self.args("}")
                a = ("brace", a, args)
            elif self.at_op(".") and self.peek(1).kind in ("id", "kw"):
                self.next()
                a = ("field", a, self.next().val)
            elif self.at_op(".") and self.peek(1).kind == "op" and self.peek(1).val == "(":
                self.next()
                self.next()
                e = self.expr()
                self.expect_op(")")
                a = ("dynfield", a, e)
            elif self.at_op("'", ".'"):
                self.next()
                a = ("transpose", a)
            else:
                return a

    def args(self, close):
        out = []
        while not self.at_op(close):
            if self.at_op(","):
                self.next()
                continue
            if self.at_op(":") and self._bare_colon():
                self.next()
                out.append(("colon_all",))
                continue
            out.append(self.expr())
        self.next()
        return out

    def primary(self):
        tk = self.next()
        if tk.kind == "num":
            return ("num", tk.val)
        if tk.kind == "str":
            return ("str", tk.val)
        if tk.kind == "id":
            return ("id", tk.val)
        if tk.kind == "kw" and tk.val == "end":
            return ("endval",)
        if tk.kind == "op":
            if tk.val == "(":
                e = self.expr()
                self.expect_op(")")
                return ("paren", e)
            if tk.val in ("[", "{"):
                close = "]" if tk.val == "[" else "}"
                rows, row = [], []
                while True:
                    if self.at_op(close):
                        self.next()
                        break
                    if self.at_op(";"):
                        self.next()
                        rows.append(row)
                        row = []
                        continue
                    if self.at_op(","):
                        self.next()
                        continue
                    row.append(self.expr())
                rows.append(row)
                rows = [r for r in rows if r]
                return ("matrix" if tk.val == "[" else "cell", rows)
            if tk.val == "@":
                if self.at_op("("):
                    self.next()
                    params = []
                    while not self.at_op(")"):
                        if self.at_op(","):
                            self.next()
                            continue
                        params.append(self.next().val)
                    self.next()
                    return ("lambda", params, self.expr())
                return ("handle", self.next().val)
            if tk.val == ":":
                return ("colon_all",)
        raise MatlabError("unexpected token %r on line %d" % (tk.val, tk.line))


# ---------------------------------------------------------------------------
# array helpers (MATLAB semantics on NumPy arrays of >= 2 dimensions)

def msize(v):
    """MATLAB size of a value (tuple, >= 2 entries)."""
    if isinstance(v, Char):
        return v.mshape
    if isinstance(v, (Cell, Struct)):
        return v.a.shape
    if sp.issparse(v):
        return v.shape
    if isinstance(v, Handle):
        return (1, 1)
    return v.shape


def numel(v):
    return int(np.prod(msize(v)))


def is_empty(v):
    return numel(v) == 0


def squeeze_trailing(a):
    """Drop trailing singleton dimensions beyond the second."""
    while a.ndim > 2 and a.shape[-1] == 1:
        a = a.reshape(a.shape[:-1])
    return a


def as_array(v):
    """Numeric ndarray view of a value (chars as codes, sparse densified)."""
    if isinstance(v, Char):
        return np.array([[float(ord(c)) for c in v]]) if len(v) else np.zeros((0, 0))
    if sp.issparse(v):
        return np.asarray(v.toarray())
    if isinstance(v, np.ndarray):
        return v
    if isinstance(v, (bool, int, float, np.floating, np.integer, np.bool_)):
        return np.array([[v]], dtype=np.float64 if not isinstance(v, (bool, np.bool_)) else bool)
    raise MatlabError("value of type %s where a numeric array is needed" % type(v).__name__)


def scalar(v):
    a = as_array(v)
    if a.size != 1:
        raise MatlabError("scalar expected, got size %s" % (a.shape,))
    return a.reshape(-1)[0]


def truth(v):
    """MATLAB's if/while condition: all elements non-zero and non-empty."""
    a = as_array(v)
    return a.size > 0 and bool(np.all(a != 0))


def pad_to(a, nd):
    return a.reshape(a.shape + (1,) * (nd - a.ndim)) if a.ndim < nd else a


def result_dtype(a, b, out):
    if (getattr(a, "dtype", None) == np.float32 or getattr(b, "dtype", None) == np.float32) and \
            out.dtype == np.float64:
        return out.astype(np.float32)
    return out


def elementwise(op, a, b):
    """Elementwise binary op with MATLAB's implicit expansion."""
    if sp.issparse(a) or sp.issparse(b):
        return sparse_elementwise(op, a, b)
    A, B = as_array(a), as_array(b)
    nd = max(A.ndim, B.ndim)
    A2, B2 = pad_to(A, nd), pad_to(B, nd)
    for x, y in zip(A2.shape, B2.shape):
        if x != y and x != 1 and y != 1:
            raise MatlabError("incompatible sizes %s and %s for %s" % (A.shape, B.shape, op))
    Af = A2.astype(np.float64) if A2.dtype == bool else A2
    Bf = B2.astype(np.float64) if B2.dtype == bool else B2
    with np.errstate(all="ignore"):
        if op == "+":
            r = Af + Bf
        elif op == "-":
            r = Af - Bf
        elif op == ".*":
            r = Af * Bf
        elif op == "./":
            r = Af / Bf
        elif op == ".\\":
            r = Bf / Af
        elif op == ".^":
            r = np.power(Af, Bf)
        elif op == "==":
            r = A2 == B2
        elif op == "~=":
            r = A2 != B2
        elif op == "<":
            r = A2 < B2
        elif op == "<=":
            r = A2 <= B2
        elif op == ">":
            r = A2 > B2
        elif op == ">=":
            r = A2 >= B2
        elif op == "&":
            r = (A2 != 0) & (B2 != 0)
        elif op == "|":
            r = (A2 != 0) | (B2 != 0)
        else:
            raise MatlabError("operator " + op)
    return squeeze_trailing(result_dtype(A, B, r))


def sparse_elementwise(op, a, b):
    sa, sb = sp.issparse(a), sp.issparse(b)
    if op in ("+", "-"):
        if sa and sb:
            return (a + b if op == "+" else a - b).tocsc()
        A, B = as_array(a), as_array(b)
        return elementwise(op, A, B)
    if op == ".*":
        if sa and sb:
            return a.multiply(b).tocsc()
        if sa:
            B = as_array(b)
            return (a.multiply(B) if B.size > 1 else a * float(B.reshape(-1)[0])).tocsc()
        A = as_array(a)
        return (b.multiply(A) if A.size > 1 else b * float(A.reshape(-1)[0])).tocsc()
    if op == "./" and sa and not sb and as_array(b).size == 1:
        return (a / float(as_array(b).reshape(-1)[0])).tocsc()
    r = elementwise(op, as_array(a), as_array(b))
    if op in ("==", "~=", "<", "<=", ">", ">=", "&", "|"):
        return r
    return sp.csc_matrix(r) if r.ndim == 2 else r


def mtimes(a, b):
    if numel(a) == 1 and not sp.issparse(a):
        return elementwise(".*", a, b)
    if numel(b) == 1 and not sp.issparse(b):
        return elementwise(".*", a, b)
    if sp.issparse(a) or sp.issparse(b):
        if sp.issparse(a) and sp.issparse(b):
            return (a @ b).tocsc()
        if sp.issparse(a):
            return np.asarray(a @ as_array(b))
        return np.asarray((as_array(a) @ b))
    A, B = as_array(a).astype(np.float64), as_array(b).astype(np.float64)
    if A.ndim > 2 or B.ndim > 2:
        raise MatlabError("matrix product of N-D arrays")
    if A.shape[1] != B.shape[0]:
        raise MatlabError("inner dimensions %s and %s" % (A.shape, B.shape))
    return result_dtype(as_array(a), as_array(b), A @ B)


def mldivide(a, b):
    if numel(a) == 1 and not sp.issparse(a):
        return elementwise("./", b, a)
    if sp.issparse(a):
        A = sp.csc_matrix(a)
        if sp.issparse(b):
            lu = spla.splu(A)
            B = sp.csc_matrix(b).toarray()
            return sp.csc_matrix(lu.solve(B))
        B = as_array(b).astype(np.float64)
        return spla.spsolve(A, B).reshape(B.shape)
    A = as_array(a).astype(np.float64)
    B = as_array(b).astype(np.float64) if not sp.issparse(b) else b.toarray()
    if A.shape[0] == A.shape[1]:
        return np.linalg.solve(A, B)
    return np.linalg.lstsq(A, B, rcond=None)[0]


def mrdivide(a, b):
    if numel(b) == 1 and not sp.issparse(b):
        return elementwise("./", a, b)
    return mldivide(transpose(b), transpose(a)).T


def transpose(v):
    if isinstance(v, Cell):
        return Cell(v.a.T)
    if isinstance(v, Struct):
        return Struct(v.a.T, v.fields)
    if sp.issparse(v):
        return v.T.tocsc()
    A = as_array(v)
    if A.ndim > 2:
        raise MatlabError("transpose of an N-D array")
    return A.T.copy()


def colon(a, b, c=None):
    """a:b or a:step:c."""
    a = float(scalar(a))
    if c is None:
        step, stop = 1.0, float(scalar(b))
    else:
        step, stop = float(scalar(b)), float(scalar(c))
    if step == 0 or (step > 0 and a > stop) or (step < 0 and a < stop):
        return np.zeros((1, 0))
    k = int(math.floor((stop - a) / step + 1e-10))
    return (a + step * np.arange(k + 1)).reshape(1, -1)


# -- index conversion -------------------------------------------------------

class _All:
    pass


ALL = _All()


def index_vector(v, n_dim):
    """0-based int vector for one subscript (':' -> all of n_dim);
    returns (ints, the subscript's MATLAB shape)."""
    if v is ALL:
        return np.arange(n_dim), (n_dim, 1)
    if sp.issparse(v):
        v = v.toarray()
    a = as_array(v)
    if a.dtype == bool:
        return np.nonzero(a.reshape(-1, order="F"))[0], a.shape
    f = a.reshape(-1, order="F")
    if f.size and (np.any(f != np.floor(f)) or np.any(f < 1)):
        raise MatlabError("subscript indices must be real positive integers")
    return f.astype(np.int64) - 1, a.shape


def is_vec(shape):
    return len(shape) == 2 and (shape[0] == 1 or shape[1] == 1)


def linear_shape(base_shape, idx_shape, k, logical):
    """Shape of A(I) for linear indexing."""
    if logical:
        if len(base_shape) == 2 and base_shape[0] == 1 and is_vec(idx_shape):
            return (1, k)
        return (k, 1)
    if is_vec(base_shape) and is_vec(idx_shape) and np.prod(base_shape) > 1 and len(idx_shape) == 2:
        return (1, k) if base_shape[0] == 1 else (k, 1)
    return tuple(idx_shape)


def reshape_f(a, shape):
    return np.reshape(a, shape, order="F")


def index_get(base, subs):
    """base(subs...) for arrays, chars, cells (paren), structs and sparse."""
    if sp.issparse(base):
        A = base.tocsr()
        if len(subs) == 1:
            dense = base.toarray()
            return index_get(dense, subs)
        r, _ = index_vector(subs[0], A.shape[0])
        c, _ = index_vector(subs[1], A.shape[1])
        return A[r][:, c].tocsc()
    if isinstance(base, Char):
        arr = np.array([list(base)], dtype=object) if len(base) else np.empty((0, 0), dtype=object)
        out = index_get_obj(arr, subs)
        return Char("".join(out.reshape(-1, order="F")))
    if isinstance(base, Cell):
        return Cell(index_get_obj(base.a, subs))
    if isinstance(base, Struct):
        return Struct(index_get_obj(base.a, subs), base.fields)
    if isinstance(base, Handle):
        raise MatlabError("indexing a function handle")
    return index_get_obj(as_array(base), subs)


def index_get_obj(A, subs):
    shape = A.shape
    if len(subs) == 0:
        return A
    if len(subs) == 1:
        s = subs[0]
        flat = A.reshape(-1, order="F")
        idx, ishape = index_vector(s, flat.size)
        logical = s is not ALL and not isinstance(s, Cell) and as_array(s).dtype == bool \
            if s is not ALL else False
        if idx.size and idx.max() >= flat.size:
            raise MatlabError("index %d exceeds %d elements" % (idx.max() + 1, flat.size))
        if s is ALL:
            return flat.reshape(-1, 1).copy()
        out_shape = linear_shape(shape, ishape, idx.size, logical)
        return reshape_f(flat[idx], out_shape)
    k = len(subs)
    if A.ndim > k:
        A = reshape_f(A, shape[:k - 1] + (int(np.prod(shape[k - 1:])),))
    elif A.ndim < k:
        A = A.reshape(A.shape + (1,) * (k - A.ndim))
    ids = []
    for d, s in enumerate(subs):
        idx, _ = index_vector(s, A.shape[d])
        if idx.size and idx.max() >= A.shape[d]:
            raise MatlabError("index %d exceeds dimension %d of size %d" % (idx.max() + 1, d + 1, A.shape[d]))
        ids.append(idx)
    out = A[np.ix_(*ids)]
    return squeeze_trailing(out)


def grow(A, new_shape, fill):
    if tuple(new_shape) == A.shape:
        return A
    B = np.empty(new_shape, dtype=A.dtype)
    if A.dtype == object:
        for k in np.ndindex(B.shape):
            B[k] = fill() if callable(fill) else fill
    else:
        B[...] = fill
    if A.size:
        B[tuple(slice(0, s) for s in A.shape)] = A
    return B


def index_set(base, subs, val, fill=0.0):
    """base(subs...) = val, returning the new value (growth, scalar expansion,
    deletion with [])."""
    is_cell, is_struct, is_char = isinstance(base, Cell), isinstance(base, Struct), isinstance(base, Char)
    if sp.issparse(base):
        return sparse_set(base, subs, val)
    delete = (not isinstance(val, (Cell, Struct, Char))) and not sp.issparse(val) and \
        isinstance(val, np.ndarray) and val.shape == (0, 0) and val.dtype != object and not is_cell
    if is_cell:
        A = base.a
        if isinstance(val, Cell):
            V = val.a
        else:
            raise MatlabError("conversion to cell from %s is not possible" % type(val).__name__)
        fillf = empty_double
    elif is_struct:
        A = base.a
        if not isinstance(val, Struct):
            if isinstance(val, np.ndarray) and val.size == 0:
                V = np.empty((0, 0), dtype=object)
                delete = True
            else:
                raise MatlabError("assigning a non-struct into a struct array")
        else:
            V = val.a
        fillf = dict
    elif is_char:
        A = np.array([list(base)], dtype=object) if len(base) else np.empty((0, 0), dtype=object)
        V = np.array([list(val)], dtype=object) if isinstance(val, Char) else as_array(val)
        fillf = "\0"
    else:
        A = as_array(base)
        V = as_array(val) if not sp.issparse(val) else val.toarray()
        fillf = fill
    if delete:
        return index_delete(base, A, subs)
    if not (is_cell or is_struct or is_char):
        if A.size == 0 and A.dtype != V.dtype:
            A = A.astype(V.dtype if V.dtype != bool else np.float64)
            if V.dtype == bool and A.size == 0:
                A = A.astype(np.float64)
        elif A.dtype == bool and V.dtype != bool:
            A = A.astype(np.float64)
        elif A.dtype == np.float64 and V.dtype == bool:
            V = V.astype(np.float64)
        elif A.dtype == np.float32:
            V = V.astype(np.float32)
        else:
            A = A.copy()
    else:
        A = A.copy()
    if len(subs) == 1:
        s = subs[0]
        n0 = A.size
        if s is ALL:
            idx = np.arange(n0)
        else:
            a = as_array(s)
            if a.dtype == bool:
                idx = np.nonzero(a.reshape(-1, order="F"))[0]
            else:
                idx, _ = index_vector(s, n0)
        need = int(idx.max()) + 1 if idx.size else 0
        if need > n0:
            if A.ndim == 2 and (A.shape[0] == 1 or A.size == 0) and not (A.shape[0] > 1):
                A = grow(A, (1, need), fillf) if A.shape[0] <= 1 else A
            elif A.ndim == 2 and A.shape[1] == 1:
                A = grow(A, (need, 1), fillf)
            else:
                raise MatlabError("linear index out of bounds for a matrix")
        flat = A.reshape(-1, order="F").copy()
        if V.size == 1:
            if flat.dtype == object:
                for k in idx:
                    flat[k] = V.reshape(-1)[0]
            else:
                flat[idx] = V.reshape(-1)[0]
        else:
            if V.size != idx.size:
                raise MatlabError("%d elements assigned to %d positions" % (V.size, idx.size))
            vf = V.reshape(-1, order="F")
            if flat.dtype == object:
                for k, x in zip(idx, vf):
                    flat[k] = x
            else:
                flat[idx] = vf
        A = reshape_f(flat, A.shape)
    else:
        k = len(subs)
        shape = list(A.shape)
        merged = A.ndim > k
        if merged:
            A = reshape_f(A, tuple(shape[:k - 1]) + (int(np.prod(shape[k - 1:])),))
        elif A.ndim < k:
            A = A.reshape(A.shape + (1,) * (k - A.ndim))
        ids = []
        new_shape = list(A.shape)
        for d, s in enumerate(subs):
            if s is ALL:
                n_d = A.shape[d]
                if A.size == 0 and n_d == 0:
                    # x(:, j) = column into an empty array takes the value's extent
                    vs = pad_to(V, k).shape if V.size > 1 else (1,) * k
                    n_d = vs[d]
                    new_shape[d] = n_d
                idx = np.arange(n_d)
            else:
                a = as_array(s)
                if a.dtype == bool:
                    idx = np.nonzero(a.reshape(-1, order="F"))[0]
                else:
                    idx, _ = index_vector(s, A.shape[d])
            if idx.size:
                new_shape[d] = max(new_shape[d], int(idx.max()) + 1)
            ids.append(idx)
        A = grow(A, tuple(new_shape), fillf)
        target = (tuple(len(i) for i in ids))
        if A.dtype == object:
            pos = list(zip(*[g.reshape(-1, order="F") for g in np.meshgrid(*ids, indexing="ij")])) \
                if all(len(i) for i in ids) else []
            vf = V.reshape(-1, order="F")
            if V.size != 1 and V.size != len(pos):
                raise MatlabError("assignment dimension mismatch: %s into %s" % (V.shape, target))
            for q, p in enumerate(pos):
                A[p] = vf[0] if V.size == 1 else vf[q]
        elif V.size == 1:
            A[np.ix_(*ids)] = V.reshape(-1)[0]
        else:
            if V.size != int(np.prod(target)):
                raise MatlabError("assignment dimension mismatch: %s into %s" % (V.shape, target))
            A[np.ix_(*ids)] = reshape_f(V, target)
        if merged and A.shape[k - 1] == int(np.prod(shape[k - 1:])):
            A = reshape_f(A, tuple(A.shape[:k - 1]) + tuple(shape[k - 1:]))   # trailing dims kept
        A = squeeze_trailing(A)
    if is_cell:
        return Cell(A)
    if is_struct:
        return Struct(A, list(base.fields) + [f for f in (val.fields if isinstance(val, Struct) else [])
                                              if f not in base.fields])
    if is_char:
        return Char("".join(str(x) for x in A.reshape(-1, order="F")))
    return A


def index_delete(base, A, subs):
    if len(subs) == 1:
        idx, _ = index_vector(subs[0], A.size)
        keep = np.ones(A.size, bool)
        keep[idx] = False
        flat = A.reshape(-1, order="F")[keep]
        out = flat.reshape(-1, 1) if (A.ndim == 2 and A.shape[1] == 1 and A.shape[0] != 1) else flat.reshape(1, -1)
    else:
        dims = [d for d, s in enumerate(subs) if s is not ALL]
        if len(dims) != 1:
            raise MatlabError("deletion needs exactly one non-colon subscript")
        d = dims[0]
        idx, _ = index_vector(subs[d], A.shape[d])
        keep = np.ones(A.shape[d], bool)
        keep[idx] = False
        out = np.compress(keep, A, axis=d)
    if isinstance(base, Cell):
        return Cell(out)
    if isinstance(base, Struct):
        return Struct(out, base.fields)
    return out


def sparse_set(base, subs, val):
    A = base.tolil()
    if len(subs) != 2:
        raise MatlabError("linear assignment into a sparse matrix")
    r, _ = index_vector(subs[0], A.shape[0])
    c, _ = index_vector(subs[1], A.shape[1])
    V = val.toarray() if sp.issparse(val) else as_array(val)
    if V.size == 1:
        V = np.full((r.size, c.size), float(V.reshape(-1)[0]))
    A[np.ix_(r, c)] = reshape_f(V, (r.size, c.size))
    return A.tocsc()


def concat(rows):
    """[a, b; c, d] for numeric, char, cell and struct values."""
    out_rows = []
    for row in rows:
        items = [x for x in row if not (isinstance(x, np.ndarray) and x.shape == (0, 0) and x.dtype != object)]
        if not items:
            continue
        if all(isinstance(x, Char) for x in items):
            out_rows.append(Char("".join(items)))
            continue
        if any(isinstance(x, Cell) for x in items):
            arrs = [x.a if isinstance(x, Cell) else Cell(np.array([[x]], dtype=object)).a for x in items]
            arrs = [a for a in arrs if a.size]
            out_rows.append(Cell(np.concatenate(arrs, axis=1) if arrs else np.empty((0, 0), object)))
            continue
        if any(isinstance(x, Struct) for x in items):
            out_rows.append(Struct(np.concatenate([x.a for x in items], axis=1), items[0].fields))
            continue
        if any(sp.issparse(x) for x in items):
            out_rows.append(sp.hstack([x if sp.issparse(x) else sp.csc_matrix(as_array(x)) for x in items]).tocsc())
            continue
        arrs = [as_array(x) for x in items]
        nd = max(a.ndim for a in arrs)
        arrs = [pad_to(a, nd) for a in arrs]
        dt = np.float32 if any(a.dtype == np.float32 for a in arrs) else \
            (bool if all(a.dtype == bool for a in arrs) else np.float64)
        out_rows.append(np.concatenate([a.astype(dt) for a in arrs], axis=1))
    if not out_rows:
        return np.zeros((0, 0))
    if len(out_rows) == 1:
        return out_rows[0]
    if all(isinstance(x, Char) for x in out_rows):
        if len(set(len(x) for x in out_rows)) != 1:
            raise MatlabError("vertical concatenation of chars of different lengths")
        raise MatlabError("char matrices are not supported")
    if any(isinstance(x, Cell) for x in out_rows):
        return Cell(np.concatenate([x.a for x in out_rows], axis=0))
    if any(isinstance(x, Struct) for x in out_rows):
        return Struct(np.concatenate([x.a for x in out_rows], axis=0), out_rows[0].fields)
    if any(sp.issparse(x) for x in out_rows):
        return sp.vstack([x if sp.issparse(x) else sp.csc_matrix(as_array(x)) for x in out_rows]).tocsc()
    arrs = [as_array(x) for x in out_rows]
    nd = max(a.ndim for a in arrs)
    arrs = [pad_to(a, nd) for a in arrs]
    dt = np.float32 if any(a.dtype == np.float32 for a in arrs) else \
        (bool if all(a.dtype == bool for a in arrs) else np.float64)
    return np.concatenate([a.astype(dt) for a in arrs], axis=0)


# ---------------------------------------------------------------------------
# interpreter

class _Break(Exception):
    pass


class _Continue(Exception):
    pass


class _Return(Exception):
    pass


class Frame:
    def __init__(self, file_funcs, nargin, nargout, name=""):
        self.name = name
        self.vars = {}
        self.file_funcs = file_funcs
        self.nargin = nargin
        self.nargout = nargout


class Interp:
    """Runs MATLAB functions from source directories (searched in order)."""

    def __init__(self, paths, stubs=None, output=None):
        self.paths = list(paths)
        self.files = {}
        self.stubs = dict(stubs or {})
        self.output = output            # callable for printed text, None = discard
        self.end_stack = []

    # -- function lookup -----------------------------------------------------
    def load_file(self, name):
        if name in self.files:
            return self.files[name]
        for d in self.paths:
            p = os.path.join(d, name + ".m")
            if os.path.exists(p):
                with open(p, encoding="utf-8", errors="replace") as f:
                    src = f.read()
                funcs, order = Parser(lex(src)).parse_file()
                entry = funcs[order[0]]
                self.files[name] = (entry, funcs)
                return self.files[name]
        self.files[name] = None
        return None

    def call(self, name, args, nargout=1, frame=None):
        """Call a function by name: subfunction of the calling file, a file on
        the path, a stub, then a built-in."""
        if frame is not None and name in frame.file_funcs:
            return self.call_user(frame.file_funcs[name], frame.file_funcs, args, nargout)
        if name in self.stubs:
            return self.stubs[name](self, args, nargout)
        f = self.load_file(name)
        if f is not None:
            entry, funcs = f
            return self.call_user(entry, funcs, args, nargout)
        if name in BUILTINS:
            out = BUILTINS[name](self, [a for a in args], nargout)
            return out if isinstance(out, list) else [out]
        raise MatlabError("undefined function or variable '%s'" % name)

    def exists_function(self, name, frame):
        return (frame is not None and name in frame.file_funcs) or name in self.stubs or \
            self.load_file(name) is not None or name in BUILTINS

    def call_user(self, fdef, funcs, args, nargout):
        _, name, params, outs, body = fdef
        fr = Frame(funcs, len(args), nargout, name)
        np_ = len(params)
        has_varargin = np_ and params[-1] == "varargin"
        fixed = params[:-1] if has_varargin else params
        if len(args) > len(fixed) and not has_varargin:
            raise MatlabError("too many input arguments to %s" % name)
        for p, a in zip(fixed, args):
            if p != "~":
                fr.vars[p] = a
        if has_varargin:
            rest = args[len(fixed):]
            arr = np.empty((1, len(rest)), dtype=object)
            for i, a in enumerate(rest):
                arr[0, i] = a
            fr.vars["varargin"] = Cell(arr) if rest else Cell(np.empty((1, 0), dtype=object))
        try:
            self.run_block(body, fr)
        except _Return:
            pass
        result = []
        for k, o in enumerate(outs):
            if o == "varargout":
                vo = fr.vars.get("varargout")
                if vo is not None:
                    result.extend(list(vo.a.reshape(-1, order="F")))
                break
            if o not in fr.vars:
                if k < max(nargout, 1):
                    raise MatlabError("output argument '%s' of %s not assigned" % (o, name))
                break
            result.append(fr.vars[o])
        return result

    # -- statements ------------------------------------------------------------
    def run_block(self, stmts, fr):
        for s in stmts:
            self.run_stmt(s, fr)

    def run_stmt(self, s, fr):
        k = s[0]
        try:
            if k == "assign":
                self.assign_stmt(s, fr)
            elif k == "expr":
                e = s[1]
                if e[0] == "id" and e[1] not in fr.vars:
                    self.call(e[1], [], 0, fr)
                elif e[0] == "index" and e[1][0] == "id" and e[1][1] not in fr.vars:
                    args = self.eval_args(e[2], fr, None)
                    self.call(e[1][1], args, 0, fr)
                else:
                    self.ev(e, fr)
            elif k == "if":
                for cond, body in s[1]:
                    if truth(self.ev(cond, fr)):
                        self.run_block(body, fr)
                        break
                else:
                    self.run_block(s[2], fr)
            elif k == "for":
                rng = self.ev(s[2], fr)
                if isinstance(rng, Cell):
                    cols = [Cell(rng.a[:, j:j + 1]) for j in range(rng.a.shape[1])]
                else:
                    A = as_array(rng)
                    A2 = A.reshape(A.shape[0], -1, order="F") if A.ndim > 2 else A
                    cols = [A2[:, j:j + 1] for j in range(A2.shape[1])] if A2.size else []
                for c in cols:
                    fr.vars[s[1]] = c
                    try:
                        self.run_block(s[3], fr)
                    except _Break:
                        break
                    except _Continue:
                        continue
            elif k == "while":
                while truth(self.ev(s[1], fr)):
                    try:
                        self.run_block(s[2], fr)
                    except _Break:
                        break
                    except _Continue:
                        continue
            elif k == "switch":
                v = self.ev(s[1], fr)
                for ce, body in s[2]:
                    if self.case_match(v, self.ev(ce, fr)):
                        self.run_block(body, fr)
                        break
                else:
                    self.run_block(s[3], fr)
            elif k == "break":
                raise _Break()
            elif k == "continue":
                raise _Continue()
            elif k == "return":
                raise _Return()
            elif k == "try":
                try:
                    self.run_block(s[1], fr)
                except MatlabError as ex:
                    if s[2]:
                        fr.vars[s[2]] = Struct()
                        fr.vars[s[2]].a[0, 0]["message"] = Char(str(ex))
                    self.run_block(s[3], fr)
            elif k == "global":
                pass
            else:
                raise MatlabError("statement " + k)
        except (_Break, _Continue, _Return):
            raise
        except MatlabError as ex:                       # MATLAB-level traceback
            if getattr(ex, "_frame", None) is not fr:
                ex._frame = fr
                ex.args = (ex.args[0] + "\n  in %s line %s" % (fr.name, s[-1]),)
            raise
        except Exception as ex:                         # report the MATLAB line
            err = MatlabError("%s: %s\n  in %s line %s" % (type(ex).__name__, ex, fr.name, s[-1]))
            err._frame = fr
            raise err from ex

    @staticmethod
    def case_match(v, c):
        if isinstance(c, Cell):
            return any(Interp.case_match(v, x) for x in c.a.reshape(-1))
        if isinstance(c, Char) or isinstance(v, Char):
            return isinstance(c, Char) and isinstance(v, Char) and str(c) == str(v)
        return numel(v) == 1 and numel(c) == 1 and scalar(v) == scalar(c)

    def assign_stmt(self, s, fr):
        lhs, rhs = s[1], s[2]
        if len(lhs) == 1:
            vals = [self.ev(rhs, fr)]
        else:
            vals = self.ev_nout(rhs, fr, len(lhs))
            if len(vals) < sum(1 for x in lhs if x is not None):
                need = max(i for i, x in enumerate(lhs) if x is not None) + 1
                if len(vals) < need:
                    raise MatlabError("too many output arguments")
        for target, v in zip(lhs, vals):
            if target is not None:
                self.assign(target, v, fr)

    # -- lvalues ------------------------------------------------------------------
    def current(self, e, fr):
        """Current value of an lvalue expression, None if undefined."""
        k = e[0]
        if k == "id":
            return fr.vars.get(e[1])
        if k == "field":
            b = self.current(e[1], fr)
            if b is None or not isinstance(b, Struct) or b.a.size != 1:
                return None
            return b.a.reshape(-1)[0].get(e[2])
        if k == "brace":
            b = self.current(e[1], fr)
            if b is None or not isinstance(b, Cell):
                return None
            subs = self.eval_args(e[2], fr, b)
            try:
                v = index_get(b, subs)
            except MatlabError:
                return None
            return v.a.reshape(-1)[0] if v.a.size == 1 else None
        if k == "index":
            b = self.current(e[1], fr)
            if b is None:
                return None
            subs = self.eval_args(e[2], fr, b)
            try:
                return index_get(b, subs)
            except MatlabError:
                return None
        raise MatlabError("invalid assignment target")

    def assign(self, e, v, fr):
        k = e[0]
        if k == "id":
            fr.vars[e[1]] = v
            return
        if k == "paren":
            return self.assign(e[1], v, fr)
        if k == "field":
            b = self.current(e[1], fr)
            if b is None or (isinstance(b, np.ndarray) and b.size == 0):
                b = Struct()
            if not isinstance(b, Struct):
                raise MatlabError("field assignment to a non-struct")
            b = b.copy()
            if b.a.size != 1:
                raise MatlabError("field assignment to a struct array")
            b.a.reshape(-1)[0][e[2]] = v
            if e[2] not in b.fields:
                b.fields.append(e[2])
            return self.assign(e[1], b, fr)
        if k == "index":
            b = self.current(e[1], fr)
            if b is None:
                b = Struct(np.empty((0, 0), dtype=object)) if isinstance(v, Struct) else \
                    (Cell(np.empty((0, 0), dtype=object)) if isinstance(v, Cell) else np.zeros((0, 0)))
            subs = self.eval_args(e[2], fr, b)
            return self.assign(e[1], index_set(b, subs, v), fr)
        if k == "brace":
            b = self.current(e[1], fr)
            if b is None or (isinstance(b, np.ndarray) and b.size == 0):
                b = Cell(np.empty((0, 0), dtype=object))
            if not isinstance(b, Cell):
                raise MatlabError("brace assignment to a non-cell")
            subs = self.eval_args(e[2], fr, b)
            wrapped = np.empty((1, 1), dtype=object)
            wrapped[0, 0] = v
            return self.assign(e[1], index_set(b, subs, Cell(wrapped)), fr)
        raise MatlabError("invalid assignment target %s" % k)

    # -- expressions ---------------------------------------------------------------
    def eval_args(self, args, fr, base):
        """Subscripts or call arguments (comma-separated lists expanded; ':'
        -> ALL; 'end' resolved against base)."""
        out = []
        for pos, a in enumerate(args):
            if a[0] == "colon_all":
                out.append(ALL)
                continue
            self.end_stack.append((base, pos, len(args)))
            try:
                vals = self.ev_multi(a, fr)
            finally:
                self.end_stack.pop()
            out.extend(vals)
        return out

    def end_value(self):
        if not self.end_stack or self.end_stack[-1][0] is None:
            raise MatlabError("'end' outside a subscript")
        base, pos, n = self.end_stack[-1]
        shp = msize(base)
        if n == 1:
            return float(np.prod(shp))
        if pos < n - 1:
            return float(shp[pos]) if pos < len(shp) else 1.0
        return float(np.prod(shp[pos:])) if pos < len(shp) else 1.0

    def ev(self, e, fr):
        vals = self.ev_multi(e, fr)
        if len(vals) != 1:
            if not vals:
                raise MatlabError("expression produced no value")
            return vals[0]
        return vals[0]

    def ev_nout(self, e, fr, nout):
        """Evaluate a call (or cell/struct list) asking for nout outputs."""
        if e[0] == "index" and e[1][0] == "id" and e[1][1] not in fr.vars:
            args = self.eval_args(e[2], fr, None)
            return self.call(e[1][1], args, nout, fr)
        if e[0] == "id" and e[1] not in fr.vars:
            return self.call(e[1], [], nout, fr)
        if e[0] == "index" and e[1][0] == "id" and isinstance(fr.vars.get(e[1][1]), Handle):
            args = self.eval_args(e[2], fr, None)
            return self.call(fr.vars[e[1][1]].name, args, nout, None)
        return self.ev_multi(e, fr)

    def ev_multi(self, e, fr):
        k = e[0]
        if k == "num":
            return [np.array([[e[1]]])]
        if k == "str":
            return [Char(e[1])]
        if k == "paren":
            return [self.ev(e[1], fr)]
        if k == "endval":
            return [np.array([[self.end_value()]])]
        if k == "colon_all":
            return [ALL]
        if k == "id":
            name = e[1]
            if name in fr.vars:
                return [fr.vars[name]]
            if name == "nargin":
                return [np.array([[float(fr.nargin)]])]
            if name == "nargout":
                return [np.array([[float(fr.nargout)]])]
            out = self.call(name, [], 1, fr)
            return out[:1]
        if k == "index":
            base_e = e[1]
            if base_e[0] == "id" and base_e[1] not in fr.vars:
                args = self.eval_args(e[2], fr, None)
                out = self.call(base_e[1], args, 1, fr)
                return out[:1]
            base = self.ev(base_e, fr)
            if isinstance(base, Handle):
                args = self.eval_args(e[2], fr, None)
                return self.call(base.name, args, 1, None)[:1]
            subs = self.eval_args(e[2], fr, base)
            return [index_get(base, subs)]
        if k == "brace":
            base = self.ev(e[1], fr)
            if not isinstance(base, Cell):
                raise MatlabError("brace indexing of a non-cell")
            subs = self.eval_args(e[2], fr, base)
            sel = index_get(base, subs)
            return CSL(sel.a.reshape(-1, order="F"))
        if k == "field":
            bases = self.ev_multi(e[1], fr)
            out = CSL()
            for b in bases:
                if isinstance(b, Struct):
                    for d in b.a.reshape(-1, order="F"):
                        if e[2] not in d:
                            raise MatlabError("reference to non-existent field '%s'" % e[2])
                        out.append(d[e[2]])
                else:
                    raise MatlabError("field access '%s' of a non-struct" % e[2])
            return out
        if k == "dynfield":
            name = str(self.ev(e[2], fr))
            return self.ev_multi(("field", e[1], name), fr)
        if k == "bin":
            op = e[1]
            a = self.ev(e[2], fr)
            b = self.ev(e[3], fr)
            if op == "*":
                return [mtimes(a, b)]
            if op == "/":
                return [mrdivide(a, b)]
            if op == "\\":
                return [mldivide(a, b)]
            if op == "^":
                if numel(a) == 1 and numel(b) == 1:
                    return [elementwise(".^", a, b)]
                raise MatlabError("matrix power")
            if op in ("==", "~=") and (isinstance(a, Char) or isinstance(b, Char)):
                return [elementwise(op, as_array(a), as_array(b))]
            return [elementwise(op, a, b)]
        if k == "un":
            v = self.ev(e[2], fr)
            if e[1] == "-":
                if sp.issparse(v):
                    return [-v]
                A = as_array(v)
                return [-(A.astype(np.float64) if A.dtype == bool else A)]
            if e[1] == "+":
                return [v]
            if sp.issparse(v):
                return [as_array(v) == 0]
            return [as_array(v) == 0]
        if k == "oror":
            return [np.array([[truth(self.ev(e[1], fr)) or truth(self.ev(e[2], fr))]])]
        if k == "andand":
            return [np.array([[truth(self.ev(e[1], fr)) and truth(self.ev(e[2], fr))]])]
        if k == "transpose":
            return [transpose(self.ev(e[1], fr))]
        if k == "range":
            a = self.ev(e[1], fr)
            c = self.ev(e[3], fr)
            if e[2] is None:
                return [colon(a, c)]
            return [colon(a, self.ev(e[2], fr), c)]
        if k == "matrix":
            rows = [[v for x in row for v in self.ev_multi(x, fr)] for row in e[1]]
            return [concat(rows)]
        if k == "cell":
            rows = []
            for row in e[1]:
                items = []
                for x in row:
                    for v in self.ev_multi(x, fr):
                        if isinstance(v, Cell):
                            items.append(v)
                        else:
                            w = np.empty((1, 1), dtype=object)
                            w[0, 0] = v
                            items.append(Cell(w))
                rows.append(items)
            if not rows:
                return [Cell(np.empty((0, 0), dtype=object))]
            return [concat(rows)]
        if k == "handle":
            return [Handle(e[1])]
        raise MatlabError("expression kind " + k)


# ---------------------------------------------------------------------------
# entry point for callers

def run(interp, name, args, nargout=1):
    """Call MATLAB function `name` with Python/NumPy arguments."""
    return interp.call(name, [to_m(a) for a in args], nargout, None)


# ---------------------------------------------------------------------------
# built-in functions (documented MATLAB behaviour restated on NumPy/SciPy)

BUILTINS = {}


def builtin(*names):
    def deco(f):
        for n in names:
            BUILTINS[n] = f
        return f
    return deco


def _num(x):
    return np.array([[float(x)]])


def _bool(x):
    return np.array([[bool(x)]])


def _dims_from(args):
    """Size arguments of zeros/ones/...: (n), (m, n, ...), ([m n ...]); a
    trailing class name; returns (shape, dtype)."""
    dtype = np.float64
    if args and isinstance(args[-1], Char):
        cls = str(args[-1])
        dtype = {"double": np.float64, "single": np.float32, "logical": bool}[cls]
        args = args[:-1]
    if not args:
        return (1, 1), dtype
    if len(args) == 1:
        a = as_array(args[0]).reshape(-1)
        dims = [int(x) for x in a] if a.size > 1 else [int(a[0]), int(a[0])]
    else:
        dims = [int(scalar(x)) for x in args]
    dims = [max(d, 0) for d in dims]
    while len(dims) > 2 and dims[-1] == 1:
        dims.pop()
    return tuple(dims), dtype


@builtin("zeros")
def _zeros(ip, a, n):
    shp, dt = _dims_from(a)
    return np.zeros(shp, dtype=dt)


@builtin("ones")
def _ones(ip, a, n):
    shp, dt = _dims_from(a)
    return np.ones(shp, dtype=dt)


@builtin("true")
def _true(ip, a, n):
    shp, _ = _dims_from(a)
    return np.ones(shp, dtype=bool)


@builtin("false")
def _false(ip, a, n):
    shp, _ = _dims_from(a)
    return np.zeros(shp, dtype=bool)


@builtin("pi")
def _pi(ip, a, n):
    return _num(math.pi)


@builtin("inf", "Inf")
def _inf(ip, a, n):
    if a:
        shp, _ = _dims_from(a)
        return np.full(shp, np.inf)
    return _num(np.inf)


@builtin("nan", "NaN")
def _nan(ip, a, n):
    if a:
        shp, _ = _dims_from(a)
        return np.full(shp, np.nan)
    return _num(np.nan)


@builtin("eps")
def _eps(ip, a, n):
    return _num(np.finfo(float).eps)


@builtin("double")
def _double(ip, a, n):
    if sp.issparse(a[0]):
        return a[0].astype(np.float64)
    return as_array(a[0]).astype(np.float64)


@builtin("single")
def _single(ip, a, n):
    return as_array(a[0]).astype(np.float32)


@builtin("logical")
def _logical(ip, a, n):
    return as_array(a[0]) != 0


@builtin("size")
def _size(ip, a, n):
    s = msize(a[0])
    if len(a) > 1:
        d = int(scalar(a[1]))
        return _num(s[d - 1] if d <= len(s) else 1)
    if n <= 1:
        return np.array([[float(x) for x in s]])
    out = [_num(s[k]) if k < len(s) else _num(1) for k in range(n)]
    if n < len(s):
        out[n - 1] = _num(int(np.prod(s[n - 1:])))
    return out


@builtin("numel")
def _numel(ip, a, n):
    return _num(numel(a[0]))


@builtin("length")
def _length(ip, a, n):
    s = msize(a[0])
    return _num(0 if min(s) == 0 else max(s))


@builtin("isempty")
def _isempty(ip, a, n):
    return _bool(is_empty(a[0]))


@builtin("isvector")
def _isvector(ip, a, n):
    s = msize(a[0])
    return _bool(len(s) == 2 and (s[0] == 1 or s[1] == 1) and s[0] * s[1] >= 1)


@builtin("isscalar")
def _isscalar(ip, a, n):
    return _bool(numel(a[0]) == 1)


@builtin("iscell")
def _iscell(ip, a, n):
    return _bool(isinstance(a[0], Cell))


@builtin("isstruct")
def _isstruct(ip, a, n):
    return _bool(isinstance(a[0], Struct))


@builtin("ischar")
def _ischar(ip, a, n):
    return _bool(isinstance(a[0], Char))


@builtin("isnumeric")
def _isnumeric(ip, a, n):
    return _bool(isinstance(a[0], np.ndarray) and a[0].dtype != bool or sp.issparse(a[0]))


@builtin("issparse")
def _issparse(ip, a, n):
    return _bool(sp.issparse(a[0]))


@builtin("isfield")
def _isfield(ip, a, n):
    s, f = a[0], a[1]
    if not isinstance(s, Struct):
        return _bool(False)
    if isinstance(f, Cell):
        return np.array([[str(x) in s.fields for x in f.a.reshape(-1)]])
    return _bool(str(f) in s.fields)


@builtin("fieldnames")
def _fieldnames(ip, a, n):
    s = a[0]
    arr = np.empty((len(s.fields), 1), dtype=object)
    for i, f in enumerate(s.fields):
        arr[i, 0] = Char(f)
    return Cell(arr)


@builtin("setfield")
def _setfield(ip, a, n):
    s = a[0].copy() if isinstance(a[0], Struct) else Struct()
    s.a.reshape(-1)[0][str(a[1])] = a[2]
    if str(a[1]) not in s.fields:
        s.fields.append(str(a[1]))
    return s


@builtin("getfield")
def _getfield(ip, a, n):
    return a[0].a.reshape(-1)[0][str(a[1])]


def _elementwise_fn(f):
    def g(ip, a, n):
        v = a[0]
        if sp.issparse(v):
            r = v.copy()
            r.data = f(r.data)
            return r
        A = as_array(v)
        with np.errstate(all="ignore"):
            return f(A.astype(np.float64) if A.dtype == bool else A)
    return g


for _name, _f in (("abs", np.abs), ("sqrt", np.sqrt), ("exp", np.exp), ("log", np.log), ("sin", np.sin),
                  ("cos", np.cos), ("floor", np.floor), ("ceil", np.ceil), ("tan", np.tan),
                  ("atan", np.arctan), ("sign", np.sign), ("log10", np.log10)):
    BUILTINS[_name] = _elementwise_fn(_f)


@builtin("round")
def _round(ip, a, n):
    A = as_array(a[0])
    return np.sign(A) * np.floor(np.abs(A) + 0.5)          # half away from zero


@builtin("atan2")
def _atan2(ip, a, n):
    return elementwise_generic(np.arctan2, a[0], a[1])


def elementwise_generic(f, x, y):
    A, B = as_array(x), as_array(y)
    nd = max(A.ndim, B.ndim)
    return squeeze_trailing(f(pad_to(A, nd), pad_to(B, nd)))


@builtin("rem")
def _rem(ip, a, n):
    return elementwise_generic(np.fmod, a[0], a[1])


@builtin("mod")
def _mod(ip, a, n):
    def f(x, y):
        with np.errstate(all="ignore"):
            r = x - np.floor(x / y) * y
        return np.where(y == 0, x, r)
    return elementwise_generic(f, a[0], a[1])


@builtin("isinf")
def _isinf(ip, a, n):
    return np.isinf(as_array(a[0]))


@builtin("isnan")
def _isnan(ip, a, n):
    return np.isnan(as_array(a[0]))


@builtin("isfinite")
def _isfinite(ip, a, n):
    return np.isfinite(as_array(a[0]))


def _first_dim(shape):
    for d, s in enumerate(shape):
        if s != 1:
            return d
    return 0


def _reduce(a, fn, empty_val=0.0):
    v = a[0]
    if sp.issparse(v):
        v = v.toarray()
    A = as_array(v)
    if A.dtype == bool:
        A = A.astype(np.float64)
    if len(a) > 1 and not (isinstance(a[1], Char)):
        d = int(scalar(a[1])) - 1
    else:
        if A.shape == (0, 0):
            return _num(empty_val)
        d = _first_dim(A.shape)
    if d >= A.ndim:
        return A
    return squeeze_trailing(fn(A, axis=d, keepdims=True))


@builtin("sum")
def _sum(ip, a, n):
    return _reduce(a, np.sum, 0.0)


@builtin("prod")
def _prod(ip, a, n):
    return _reduce(a, np.prod, 1.0)


@builtin("mean")
def _mean(ip, a, n):
    return _reduce(a, np.mean, np.nan)


@builtin("cumsum")
def _cumsum(ip, a, n):
    A = as_array(a[0]).astype(np.float64)
    d = int(scalar(a[1])) - 1 if len(a) > 1 else _first_dim(A.shape)
    return np.cumsum(A, axis=d)


@builtin("any")
def _any(ip, a, n):
    v = a[0].toarray() if sp.issparse(a[0]) else as_array(a[0])
    if v.size == 0:
        return _bool(False)
    d = int(scalar(a[1])) - 1 if len(a) > 1 else _first_dim(v.shape)
    return squeeze_trailing(np.any(v != 0, axis=d, keepdims=True))


@builtin("all")
def _all(ip, a, n):
    v = a[0].toarray() if sp.issparse(a[0]) else as_array(a[0])
    if v.size == 0:
        return _bool(True)
    d = int(scalar(a[1])) - 1 if len(a) > 1 else _first_dim(v.shape)
    return squeeze_trailing(np.all(v != 0, axis=d, keepdims=True))


def _minmax(a, n, which):
    fn = np.fmin if which == "min" else np.fmax
    if len(a) >= 2 and numel(a[1]) > 0:                       # elementwise min(a, b)
        return elementwise_generic(fn, a[0], a[1])
    v = a[0].toarray() if sp.issparse(a[0]) else as_array(a[0])
    if v.dtype == bool:
        v = v.astype(np.float64)
    if v.size == 0:
        return [np.zeros((0, 0)), np.zeros((0, 0))] if n > 1 else np.zeros((0, 0))
    d = int(scalar(a[2])) - 1 if len(a) >= 3 else _first_dim(v.shape)
    allnan = np.all(np.isnan(v), axis=d, keepdims=True)
    w = np.where(np.isnan(v), np.inf if which == "min" else -np.inf, v)
    idx = (np.argmin(w, axis=d) if which == "min" else np.argmax(w, axis=d))
    idx = np.expand_dims(idx, d)
    val = np.take_along_axis(v, idx, axis=d)
    val = np.where(allnan, np.nan, val)
    if n > 1:
        return [squeeze_trailing(val), squeeze_trailing(idx.astype(np.float64) + 1)]
    return squeeze_trailing(val)


@builtin("min")
def _min(ip, a, n):
    return _minmax(a, n, "min")


@builtin("max")
def _max(ip, a, n):
    return _minmax(a, n, "max")


@builtin("find")
def _find(ip, a, n):
    v = a[0].toarray() if sp.issparse(a[0]) else as_array(a[0])
    flat = v.reshape(-1, order="F")
    idx = np.nonzero(flat)[0]
    if len(a) > 1:
        idx = idx[:int(scalar(a[1]))]
    if n >= 2:
        r = (idx % v.shape[0]).astype(np.float64) + 1
        c = (idx // v.shape[0]).astype(np.float64) + 1
        return [r.reshape(-1, 1), c.reshape(-1, 1)]
    out = idx.astype(np.float64) + 1
    if v.ndim == 2 and v.shape[0] == 1 and v.shape[1] != 1:
        return out.reshape(1, -1)
    if v.size == 0 or (v.ndim == 2 and v.shape == (1, 1) and idx.size == 0):
        return np.zeros((1, 0)) if v.ndim == 2 and v.shape[0] == 1 else np.zeros((0, 1))
    return out.reshape(-1, 1)


@builtin("nnz")
def _nnz(ip, a, n):
    v = a[0]
    return _num(v.count_nonzero() if sp.issparse(v) else np.count_nonzero(as_array(v)))


def _sort_array(A, d, descend):
    """Stable sort along axis d; NaNs last for ascending (MATLAB)."""
    key = -A if descend else A
    idx = np.argsort(key, axis=d, kind="stable")
    return np.take_along_axis(A, idx, axis=d), idx


@builtin("sort")
def _sort(ip, a, n):
    v = a[0]
    if isinstance(v, Cell):
        items = [str(x) for x in v.a.reshape(-1, order="F")]
        order = sorted(range(len(items)), key=lambda k: items[k])
        arr = np.empty(v.a.shape, dtype=object)
        flat = arr.reshape(-1, order="F")
        for k, o in enumerate(order):
            flat[k] = Char(items[o])
        out = Cell(reshape_f(flat, v.a.shape))
        return [out, np.array(order, float).reshape(v.a.shape, order="F") + 1] if n > 1 else out
    was_sparse = sp.issparse(v)
    A = v.toarray() if was_sparse else as_array(v)
    d = _first_dim(A.shape)
    descend = False
    for x in a[1:]:
        if isinstance(x, Char):
            descend = str(x).lower() == "descend"
        else:
            d = int(scalar(x)) - 1
    B, idx = _sort_array(A, d, descend)
    if was_sparse:
        B = sp.csc_matrix(B)
    if n > 1:
        return [B, idx.astype(np.float64) + 1]
    return B


@builtin("sortrows")
def _sortrows(ip, a, n):
    A = as_array(a[0])
    order = np.lexsort([A[:, j] for j in range(A.shape[1] - 1, -1, -1)]) if A.size else np.zeros(0, int)
    B = A[order]
    if n > 1:
        return [B, order.astype(np.float64).reshape(-1, 1) + 1]
    return B


@builtin("unique")
def _unique(ip, a, n):
    v = a[0]
    rows = any(isinstance(x, Char) and str(x) == "rows" for x in a[1:])
    if isinstance(v, Cell):
        items = [str(x) for x in v.a.reshape(-1, order="F")]
        uniq = sorted(set(items))
        arr = np.empty((len(uniq), 1), dtype=object)
        for k, s in enumerate(uniq):
            arr[k, 0] = Char(s)
        out = Cell(arr)
        if v.a.shape[0] == 1 and v.a.ndim == 2 and v.a.shape[1] > 1:
            out = Cell(arr.T)
        if n > 1:
            ia = np.array([items.index(s) for s in uniq], float).reshape(-1, 1) + 1
            ic = np.array([uniq.index(s) for s in items], float).reshape(-1, 1) + 1
            return [out, ia, ic]
        return out
    A = as_array(v)
    if rows:
        if A.size == 0:
            return [A, np.zeros((0, 1)), np.zeros((0, 1))] if n > 1 else A
        order = np.lexsort([A[:, j] for j in range(A.shape[1] - 1, -1, -1)])
        S = A[order]
        first = np.ones(S.shape[0], bool)
        first[1:] = np.any(S[1:] != S[:-1], axis=1)
        C = S[first]
        grp = np.cumsum(first) - 1
        ic = np.empty(A.shape[0], np.int64)
        ic[order] = grp
        ia = order[first]
        if n > 1:
            return [C, ia.astype(float).reshape(-1, 1) + 1, ic.astype(float).reshape(-1, 1) + 1]
        return C
    flat = A.reshape(-1, order="F")
    C, ia, ic = np.unique(flat, return_index=True, return_inverse=True)
    if A.ndim == 2 and A.shape[0] == 1 and A.shape[1] >= 1:
        out = C.reshape(1, -1)
    else:
        out = C.reshape(-1, 1)
    if n > 1:
        return [out, ia.astype(float).reshape(-1, 1) + 1, ic.astype(float).reshape(-1, 1) + 1]
    return out


@builtin("ismember")
def _ismember(ip, a, n):
    x, s = a[0], a[1]
    if isinstance(x, (Cell, Char)) or isinstance(s, (Cell, Char)):
        xs = [str(e) for e in x.a.reshape(-1, order="F")] if isinstance(x, Cell) else [str(x)]
        ss = [str(e) for e in s.a.reshape(-1, order="F")] if isinstance(s, Cell) else [str(s)]
        pos = {}
        for k, e in enumerate(ss):
            pos.setdefault(e, k + 1)
        tf = np.array([e in pos for e in xs])
        loc = np.array([pos.get(e, 0) for e in xs], float)
        shape = x.a.shape if isinstance(x, Cell) else (1, 1)
        tf, loc = reshape_f(tf, shape), reshape_f(loc, shape)
        return [tf, loc] if n > 1 else tf
    X, S = as_array(x), as_array(s)
    sf = S.reshape(-1, order="F")
    pos = {}
    for k, e in enumerate(sf):
        pos.setdefault(float(e), k + 1)
    xf = X.reshape(-1, order="F")
    tf = np.array([float(e) in pos for e in xf], dtype=bool)
    loc = np.array([pos.get(float(e), 0) for e in xf], float)
    tf, loc = reshape_f(tf, X.shape), reshape_f(loc, X.shape)
    return [tf, loc] if n > 1 else tf


@builtin("strcmp", "strcmpi")
def _strcmp(ip, a, n, ci=False):
    def norm(s):
        return str(s).lower() if ci else str(s)
    x, y = a[0], a[1]
    if isinstance(x, Cell) or isinstance(y, Cell):
        cellv, other = (x, y) if isinstance(x, Cell) else (y, x)
        if isinstance(other, Cell):
            return np.vectorize(lambda p, q: isinstance(p, Char) and isinstance(q, Char) and norm(p) == norm(q),
                                otypes=[bool])(cellv.a, other.a)
        return np.vectorize(lambda p: isinstance(p, Char) and isinstance(other, Char) and norm(p) == norm(other),
                            otypes=[bool])(cellv.a)
    return _bool(isinstance(x, Char) and isinstance(y, Char) and norm(x) == norm(y))


BUILTINS["strcmpi"] = lambda ip, a, n: _strcmp(ip, a, n, ci=True)


@builtin("str2func")
def _str2func(ip, a, n):
    return Handle(str(a[0]))


@builtin("func2str")
def _func2str(ip, a, n):
    return Char(a[0].name)


@builtin("feval")
def _feval(ip, a, n):
    f = a[0]
    name = f.name if isinstance(f, Handle) else str(f)
    return ip.call(name, a[1:], max(n, 1), None)


@builtin("str2num", "str2double")
def _str2num(ip, a, n):
    try:
        return _num(float(str(a[0]).strip()))
    except ValueError:
        return np.zeros((0, 0))


@builtin("num2str")
def _num2str(ip, a, n):
    v = scalar(a[0])
    return Char(("%d" % v) if float(v).is_integer() else ("%.4g" % v))


def _mformat(fmt, vals):
    fmt = str(fmt).replace("\\n", "\n").replace("\\t", "\t")
    fmt = re.sub(r"%(-?\d*)i", r"%\1d", fmt)
    flat = []
    for v in vals:
        if isinstance(v, Char):
            flat.append(str(v))
        else:
            flat.extend(float(x) for x in as_array(v).reshape(-1, order="F"))
    conv = []
    specs = re.findall(r"%[-+ #0]*\d*(?:\.\d+)?([diouxXeEfgGcs])", fmt)
    for k, s in enumerate(specs):
        if k < len(flat):
            x = flat[k]
            conv.append(int(x) if s in "diouxX" and not isinstance(x, str) else x)
    try:
        return fmt % tuple(conv) if specs else fmt
    except (TypeError, ValueError):
        return fmt


@builtin("sprintf")
def _sprintf(ip, a, n):
    return Char(_mformat(a[0], a[1:]))


@builtin("fprintf", "disp", "display", "warning")
def _fprintf(ip, a, n):
    if ip.output is not None and a:
        ip.output(_mformat(a[0], a[1:]) if isinstance(a[0], Char) else str(a[0]))
    return []


@builtin("error")
def _error(ip, a, n):
    if not a:
        return []
    args = a[1:] if len(a) > 1 and isinstance(a[0], Char) and re.match(r"^\w+(:\w+)+$", str(a[0])) else a
    raise MatlabError(_mformat(args[0], args[1:]))


@builtin("upper")
def _upper(ip, a, n):
    return Char(str(a[0]).upper())


@builtin("lower")
def _lower(ip, a, n):
    return Char(str(a[0]).lower())


@builtin("linspace")
def _linspace(ip, a, n):
    d1, d2 = float(scalar(a[0])), float(scalar(a[1]))
    k = int(math.floor(scalar(a[2]))) if len(a) > 2 else 100
    if k < 1:
        return np.zeros((1, 0))
    if k == 1:
        return np.array([[d2]])
    n1 = k - 1
    y = d1 + np.arange(k) * ((d2 - d1) / n1)
    y[-1] = d2
    return y.reshape(1, -1)


@builtin("meshgrid")
def _meshgrid(ip, a, n):
    x = as_array(a[0]).reshape(-1, order="F")
    y = as_array(a[1]).reshape(-1, order="F") if len(a) > 1 else x
    X, Y = np.meshgrid(x, y)
    return [X, Y] if n > 1 else X


@builtin("repmat")
def _repmat(ip, a, n):
    v = a[0]
    if len(a) == 2:
        reps = [int(x) for x in as_array(a[1]).reshape(-1)]
        if len(reps) == 1:
            reps = reps * 2
    else:
        reps = [int(scalar(x)) for x in a[1:]]
    if isinstance(v, Cell):
        A = v.a
        A = pad_to(A, len(reps))
        return Cell(np.tile(A, reps + [1] * (A.ndim - len(reps))))
    A = as_array(v)
    nd = max(A.ndim, len(reps))
    A = pad_to(A, nd)
    reps = reps + [1] * (nd - len(reps))
    return squeeze_trailing(np.tile(A, reps))


@builtin("reshape")
def _reshape(ip, a, n):
    v = a[0]
    if len(a) == 2:
        dims = [int(x) for x in as_array(a[1]).reshape(-1)]
    else:
        dims = [(-1 if numel(x) == 0 else int(scalar(x))) for x in a[1:]]
    if isinstance(v, Cell):
        return Cell(reshape_f(v.a, dims))
    if sp.issparse(v):
        v = v.toarray()
        return sp.csc_matrix(reshape_f(v, dims))
    return squeeze_trailing(reshape_f(as_array(v), dims))


@builtin("permute")
def _permute(ip, a, n):
    order = [int(x) - 1 for x in as_array(a[1]).reshape(-1)]
    v = a[0]
    A = v.a if isinstance(v, Cell) else as_array(v)
    A = pad_to(A, len(order))
    out = squeeze_trailing(np.transpose(A, order))
    return Cell(out) if isinstance(v, Cell) else out


@builtin("squeeze")
def _squeeze(ip, a, n):
    A = as_array(a[0])
    if A.ndim <= 2:
        return A
    s = [x for x in A.shape if x != 1]
    while len(s) < 2:
        s.append(1)
    return A.reshape(s, order="F")


@builtin("cat")
def _cat(ip, a, n):
    d = int(scalar(a[0])) - 1
    arrs = [as_array(x) for x in a[1:]]
    nd = max(max(x.ndim for x in arrs), d + 1)
    arrs = [pad_to(x, nd) for x in arrs]
    return squeeze_trailing(np.concatenate(arrs, axis=d))


@builtin("horzcat")
def _horzcat(ip, a, n):
    return concat([list(a)])


@builtin("vertcat")
def _vertcat(ip, a, n):
    return concat([[x] for x in a])


@builtin("fliplr")
def _fliplr(ip, a, n):
    return as_array(a[0])[:, ::-1].copy()


@builtin("flipud")
def _flipud(ip, a, n):
    return as_array(a[0])[::-1].copy()


@builtin("dot")
def _dot(ip, a, n):
    A, B = as_array(a[0]), as_array(a[1])
    return _num(np.sum(A.reshape(-1) * B.reshape(-1)))


@builtin("norm")
def _norm(ip, a, n):
    A = as_array(a[0])
    if is_vec(A.shape):
        return _num(np.sqrt(np.sum(A * A)))
    return _num(np.linalg.norm(A, 2))


@builtin("diag")
def _diag(ip, a, n):
    v = a[0]
    if sp.issparse(v):
        if min(v.shape) == 1:
            return sp.diags(v.toarray().reshape(-1)).tocsc()
        return sp.csc_matrix(v.diagonal().reshape(-1, 1))
    A = as_array(v)
    if is_vec(A.shape):
        return np.diag(A.reshape(-1))
    return A.diagonal().reshape(-1, 1).copy()


@builtin("eye")
def _eye(ip, a, n):
    shp, _ = _dims_from(a)
    return np.eye(shp[0], shp[1])


@builtin("speye")
def _speye(ip, a, n):
    shp, _ = _dims_from(a)
    return sp.identity(shp[0], format="csc") if shp[0] == shp[1] else sp.eye(shp[0], shp[1], format="csc")


@builtin("sparse")
def _sparse(ip, a, n):
    if len(a) == 1:
        return sp.csc_matrix(as_array(a[0]).astype(np.float64))
    if len(a) == 2:
        return sp.csc_matrix((int(scalar(a[0])), int(scalar(a[1]))))
    i = as_array(a[0]).reshape(-1, order="F").astype(np.int64) - 1
    j = as_array(a[1]).reshape(-1, order="F").astype(np.int64) - 1
    v = as_array(a[2]).reshape(-1, order="F").astype(np.float64)
    if v.size == 1 and i.size > 1:
        v = np.full(i.size, v[0])
    if len(a) >= 5:
        m, nn = int(scalar(a[3])), int(scalar(a[4]))
    else:
        m = int(i.max()) + 1 if i.size else 0
        nn = int(j.max()) + 1 if j.size else 0
    M = sp.coo_matrix((v, (i, j)), shape=(m, nn)).tocsc()
    M.sum_duplicates()
    M.eliminate_zeros()
    return M


@builtin("spdiags")
def _spdiags(ip, a, n):
    B = as_array(a[0])
    d = [int(x) for x in as_array(a[1]).reshape(-1)]
    m, nn = int(scalar(a[2])), int(scalar(a[3]))
    out = sp.lil_matrix((m, nn))
    for k, dk in enumerate(d):
        col = B[:, k]
        for jcol in range(nn):
            irow = jcol - dk
            if 0 <= irow < m:
                # MATLAB takes column j's value B(j, k) for m >= n
                out[irow, jcol] = col[jcol] if m >= nn else col[irow]
    return out.tocsc()


@builtin("full")
def _full(ip, a, n):
    v = a[0]
    return np.asarray(v.toarray()) if sp.issparse(v) else v


@builtin("interp1")
def _interp1(ip, a, n):
    x = as_array(a[0]).reshape(-1, order="F").astype(np.float64)
    v = as_array(a[1]).reshape(-1, order="F").astype(np.float64)
    xq = as_array(a[2])
    method = str(a[3]).lower() if len(a) > 3 and isinstance(a[3], Char) else "linear"
    q = xq.reshape(-1, order="F").astype(np.float64)
    order = np.argsort(x, kind="stable")
    xs, vs = x[order], v[order]
    out = np.full(q.size, np.nan)
    inside = (q >= xs[0]) & (q <= xs[-1])
    if method == "nearest":
        k = np.searchsorted(xs, q[inside], side="left")
        k = np.clip(k, 1, xs.size - 1) if xs.size > 1 else np.zeros_like(k)
        if xs.size > 1:
            left, right = xs[k - 1], xs[k]
            # ties go to the larger sample (round half up)
            pick = np.where(q[inside] - left < right - q[inside], k - 1, k)
        else:
            pick = k
        out[inside] = vs[pick]
    elif method == "linear":
        out[inside] = np.interp(q[inside], xs, vs)
    else:
        raise MatlabError("interp1 method " + method)
    return reshape_f(out, xq.shape)


@builtin("inpolygon")
def _inpolygon(ip, a, n):
    X, Y = as_array(a[0]), as_array(a[1])
    xv = as_array(a[2]).reshape(-1, order="F").astype(np.float64)
    yv = as_array(a[3]).reshape(-1, order="F").astype(np.float64)
    x = X.reshape(-1, order="F").astype(np.float64)
    y = Y.reshape(-1, order="F").astype(np.float64)
    if xv[0] != xv[-1] or yv[0] != yv[-1]:
        xv = np.append(xv, xv[0])
        yv = np.append(yv, yv[0])
    inside = np.zeros(x.size, bool)
    on = np.zeros(x.size, bool)
    for k in range(xv.size - 1):
        x1, y1, x2, y2 = xv[k], yv[k], xv[k + 1], yv[k + 1]
        # boundary: collinear and within the segment's box
        cross = (x2 - x1) * (y - y1) - (y2 - y1) * (x - x1)
        within = (np.minimum(x1, x2) <= x) & (x <= np.maximum(x1, x2)) & \
            (np.minimum(y1, y2) <= y) & (y <= np.maximum(y1, y2))
        on |= (cross == 0) & within
        # crossing number (half-open in y)
        cond = (y1 > y) != (y2 > y)
        with np.errstate(all="ignore"):
            xint = x1 + (y - y1) * (x2 - x1) / (y2 - y1)
        inside ^= cond & (x < xint)
    res = reshape_f(inside | on, X.shape)
    return [res, reshape_f(on, X.shape)] if n > 1 else res


@builtin("clock")
def _clock(ip, a, n):
    return np.zeros((1, 6))


@builtin("etime")
def _etime(ip, a, n):
    return _num(0.0)


@builtin("tic")
def _tic(ip, a, n):
    return [] if n == 0 else _num(0.0)


@builtin("toc")
def _toc(ip, a, n):
    return _num(0.0)


@builtin("isMATLABReleaseOlderThan")
def _release_older(ip, a, n):
    return _bool(False)                  # behave as a current release


@builtin("deal")
def _deal(ip, a, n):
    if len(a) == 1:
        return [a[0]] * max(n, 1)
    return list(a)


@builtin("cell")
def _cell(ip, a, n):
    shp, _ = _dims_from(a)
    return Cell.empty(shp)


@builtin("struct")
def _struct(ip, a, n):
    s = Struct()
    for k in range(0, len(a), 2):
        s.a[0, 0][str(a[k])] = a[k + 1]
        s.fields.append(str(a[k]))
    return s


@builtin("class")
def _class(ip, a, n):
    v = a[0]
    if isinstance(v, Char):
        return Char("char")
    if isinstance(v, Cell):
        return Char("cell")
    if isinstance(v, Struct):
        return Char("struct")
    if sp.issparse(v):
        return Char("double")
    A = as_array(v)
    return Char({np.dtype(bool): "logical", np.dtype(np.float32): "single"}.get(A.dtype, "double"))
