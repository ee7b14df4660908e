"""mlite: a small interpreter for the subset of MATLAB that the reference's
hot-path functions are written in.  TEST INFRASTRUCTURE ONLY.

It runs the reference's own ``.m`` files (``SRC/MNAD/*.m``,
``SRC/migration/Born_adj_MNAD.m``) on small inputs in this container, so the
golden fixtures under ``tests/golden/`` come from the reference code itself,
not from a restatement of it.  Neither MATLAB nor GNU Octave is available
here; this covers exactly what those files use:

* function files with several outputs and ``nargin``;
* ``for`` / ``if`` / ``elseif`` / ``else`` / ``while``;
* column-major arrays with 1-based, ``end``-relative, colon and linear
  indexing, indexed assignment that grows arrays, and ``A(:)``;
* element-wise and scalar arithmetic with implicit expansion;
* sparse ``sparse(I,J,V,m,n)`` and sparse-matrix times vector;
* cells (``data{1}``), strings, ``save`` / ``load`` into an in-memory store;
* the builtins listed in ``BUILTINS``.

Display calls (``imagesc``, ``caxis``, ``drawnow``) are accepted and do
nothing (the run is headless).  Arithmetic is IEEE double, as in MATLAB;
sparse products accumulate column by column, as a compressed-column
product does.
"""
from __future__ import annotations

import math
import os
import re

import numpy as np
import scipy.sparse as sp

# ---------------------------------------------------------------------------
# values


class Cell:
    """A cell array: items in column-major order, shape (rows, cols)."""

    def __init__(self, items=None, shape=None):
        self.items = list(items or [])
        self.shape = shape or (1, len(self.items))


class MatlabError(RuntimeError):
    def __init__(self, ident, msg):
        self.identifier = ident
        super().__init__(f"{ident}: {msg}")


def _case_match(subject, option):
    if isinstance(subject, str) or isinstance(option, str):
        return isinstance(subject, str) and isinstance(option, str) and subject == option
    return bool(np.all(num(subject) == num(option)))


def num(x):
    """Any numeric value as a 2-D float/bool array."""
    if isinstance(x, np.ndarray):
        return x if x.ndim == 2 else x.reshape(1, -1) if x.ndim <= 1 else x
    if isinstance(x, (bool, np.bool_)):
        return np.array([[bool(x)]])
    if isinstance(x, (int, float, np.integer, np.floating)):
        return np.array([[float(x)]])
    if isinstance(x, str):
        return np.array([[float(ord(c)) for c in x]])
    if sp.issparse(x):
        return x.toarray()
    raise TypeError(f"not numeric: {type(x)}")


def scalar(x):
    a = num(x)
    if a.size != 1:
        raise ValueError(f"expected a scalar, got shape {a.shape}")
    return a.flat[0]


def truth(x):
    a = num(x)
    return a.size > 0 and bool(np.all(a != 0))


# ---------------------------------------------------------------------------
# lexer

TOKEN = re.compile(r"""
    (?P<ws>[ \t]+)
  | (?P<cont>\.\.\.[^\n]*\n)
  | (?P<comment>%[^\n]*)
  | (?P<nl>\n)
  | (?P<num>(?:\d+(?:\.(?![*/^'\\])\d*)?|\.\d+)(?:[eE][+-]?\d+)?)
  | (?P<id>[A-Za-z_]\w*)
  | (?P<op>\.\^|\.\*|\./|\.'|==|~=|<=|>=|&&|\|\||[-+*/^\\<>&|~=(){}\[\],;:'@.])
""", re.VERBOSE)

KEYWORDS = {"function", "end", "for", "if", "elseif", "else", "while", "return", "break", "continue", "switch",
            "case", "otherwise"}


def lex(src):
    toks = []
    i, depth = 0, []          # depth: stack of '(' '[' '{'
    n = len(src)
    while i < n:
        c = src[i]
        if c == "'":
            prev = toks[-1] if toks else None
            transpose = prev and not prev[2] and (prev[0] in ("num", "id", "str") and prev[1] not in KEYWORDS or
                                                 prev[1] in (")", "]", "}", "'", ".'"))
            if not transpose:
                j = i + 1
                s = []
                while True:
                    if src[j] == "'" and j + 1 < n and src[j + 1] == "'":
                        s.append("'")
                        j += 2
                    elif src[j] == "'":
                        break
                    else:
                        s.append(src[j])
                        j += 1
                toks.append(("str", "".join(s), False))
                i = j + 1
                continue
        m = TOKEN.match(src, i)
        if not m:
            raise SyntaxError(f"cannot lex at {src[i:i + 30]!r}")
        kind = m.lastgroup
        text = m.group(kind)
        i = m.end()
        if kind in ("comment", "cont"):
            continue
        if kind == "ws":
            # whitespace after a token: separates elements inside [] / {} and
            # marks command syntax ("clear a b") at statement level
            if toks:
                toks[-1] = (toks[-1][0], toks[-1][1], True)
            continue
        if kind == "op":
            if text in "([{":
                depth.append(text)
            elif text in ")]}" and depth:
                depth.pop()
        if kind == "nl" and depth and depth[-1] in "[{":
            kind, text = "op", ";"
        if kind == "id" and text in KEYWORDS:
            kind = "kw"
        toks.append((kind, text, False))   # (kind, text, followed by whitespace)
    toks.append(("eof", "", False))
    return toks


# ---------------------------------------------------------------------------
# parser (AST as tuples)

class Parser:
    def __init__(self, toks):
        self.t = toks
        self.i = 0
        self.in_matrix = 0
        self.in_index = 0

    def peek(self, k=0):
        return self.t[self.i + k]

    def next(self):
        tok = self.t[self.i]
        self.i += 1
        return tok

    def accept(self, text):
        if self.peek()[1] == text and self.peek()[0] in ("op", "kw"):
            return self.next()
        return None

    def expect(self, text):
        tok = self.next()
        if tok[1] != text:
            raise SyntaxError(f"expected {text!r}, got {tok[1]!r}")
        return tok

    def skip_sep(self):
        while self.peek()[0] == "nl" or self.peek()[1] in (";", ","):
            self.next()

    # -- statements
    def file(self):
        funcs = {}
        self.skip_sep()
        while self.peek()[0] != "eof":
            f = self.function()
            funcs[f[1]] = f
            self.skip_sep()
        return funcs

    def function(self):
        self.expect("function")
        outs = []
        if self.peek()[1] == "[":
            self.next()
            while not self.accept("]"):
                tok = self.next()
                if tok[0] == "id":
                    outs.append(tok[1])
        elif self.peek(1)[1] == "=":
            outs.append(self.next()[1])
        if self.accept("="):
            pass
        name = self.next()[1]
        args = []
        if self.accept("("):
            while not self.accept(")"):
                tok = self.next()
                if tok[0] == "id":
                    args.append(tok[1])
        body = self.block(("end", "function", "eof"))
        self.accept("end")
        return ("function", name, args, outs, body)

    def block(self, stops):
        stmts = []
        while True:
            self.skip_sep()
            tok = self.peek()
            if tok[0] == "eof" or (tok[0] == "kw" and tok[1] in stops):
                return stmts
            stmts.append(self.statement())

    def statement(self):
        tok = self.peek()
        if tok[0] == "kw":
            k = tok[1]
            if k == "for":
                self.next()
                paren = self.accept("(")
                var = self.next()[1]
                self.expect("=")
                rng = self.expr()
                if paren:
                    self.expect(")")
                body = self.block(("end",))
                self.expect("end")
                return ("for", var, rng, body)
            if k == "while":
                self.next()
                cond = self.expr()
                body = self.block(("end",))
                self.expect("end")
                return ("while", cond, body)
            if k == "if":
                self.next()
                arms = []
                cond = self.expr()
                body = self.block(("elseif", "else", "end"))
                arms.append((cond, body))
                other = []
                while True:
                    if self.accept("elseif"):
                        cond = self.expr()
                        body = self.block(("elseif", "else", "end"))
                        arms.append((cond, body))
                    elif self.accept("else"):
                        other = self.block(("end",))
                    else:
                        self.expect("end")
                        break
                return ("if", arms, other)
            if k == "switch":
                self.next()
                subject = self.expr()
                cases, other = [], []
                self.skip_sep()
                while True:
                    if self.accept("case"):
                        label = self.expr()
                        cases.append((label, self.block(("case", "otherwise", "end"))))
                    elif self.accept("otherwise"):
                        other = self.block(("case", "otherwise", "end"))
                    else:
                        self.expect("end")
                        break
                return ("switch", subject, cases, other)
            if k in ("return", "break", "continue"):
                self.next()
                return (k,)
            raise SyntaxError(f"unexpected keyword {k}")
        # multiple assignment [a, b] = f(...)
        if tok[1] == "[":
            j = self.i
            depth = 0
            while True:
                t = self.t[j]
                if t[1] == "[":
                    depth += 1
                elif t[1] == "]":
                    depth -= 1
                    if depth == 0:
                        break
                j += 1
            if self.t[j + 1][1] == "=" and self.t[j + 2][1] != "=":
                self.next()
                targets = []
                while not self.accept("]"):
                    if self.accept(",") or self.accept(";"):
                        continue
                    targets.append(self.postfix())
                self.expect("=")
                return ("massign", targets, self.expr())
        # command syntax: name word word ... (e.g. "clear xz zs", "save Source Source")
        if tok[0] == "id" and tok[2] and self.peek(1)[0] in ("id", "num") and self.peek(2)[1] not in ("=", "("):
            name = self.next()[1]
            words = []
            while self.peek()[0] in ("id", "num", "kw") and self.peek()[1] not in ("end",):
                words.append(("str", self.next()[1]))
            return ("expr", ("index", ("id", name), words))
        # assignment or expression statement
        start = self.i
        if tok[0] == "id":
            target = self.postfix()
            if self.peek()[1] == "=" and self.peek(1)[1] != "=":
                self.next()
                return ("assign", target, self.expr())
            self.i = start
        # command syntax: name word (e.g. "drawnow", "hold on") -> call
        e = self.expr()
        return ("expr", e)

    # -- expressions (MATLAB precedence)
    def expr(self):
        return self.oror()

    def oror(self):
        a = self.andand()
        while self.accept("||"):
            a = ("||", a, self.andand())
        return a

    def andand(self):
        a = self.orr()
        while self.accept("&&"):
            a = ("&&", a, self.orr())
        return a

    def orr(self):
        a = self.andd()
        while self.peek()[1] == "|" and self.peek()[0] == "op":
            self.next()
            a = ("bin", "|", a, self.andd())
        return a

    def andd(self):
        a = self.cmp()
        while self.peek()[1] == "&" and self.peek()[0] == "op":
            self.next()
            a = ("bin", "&", a, self.cmp())
        return a

    def cmp(self):
        a = self.rng()
        while self.peek()[1] in ("==", "~=", "<", "<=", ">", ">=") and self.peek()[0] == "op":
            op = self.next()[1]
            a = ("bin", op, a, self.rng())
        return a

    def rng(self):
        if self.in_index and self.peek()[1] == ":" and self.peek(1)[1] in (",", ")"):
            self.next()
            return ("colon",)
        a = self.add()
        if self.peek()[1] == ":" and self.peek()[0] == "op":
            self.next()
            b = self.add()
            if self.peek()[1] == ":" and self.peek()[0] == "op":
                self.next()
                c = self.add()
                return ("range", a, b, c)
            return ("range", a, None, b)
        return a

    def _element_break(self):
        # inside [] a whitespace-separated +/- followed by no whitespace starts a new element
        prev = self.t[self.i - 1]
        tok = self.peek()
        return self.in_matrix and prev[2] and tok[1] in ("+", "-") and not tok[2]

    def add(self):
        a = self.mul()
        while self.peek()[1] in ("+", "-") and self.peek()[0] == "op" and not self._element_break():
            op = self.next()[1]
            a = ("bin", op, a, self.mul())
        return a

    def mul(self):
        a = self.unary()
        while self.peek()[1] in ("*", "/", ".*", "./", "\\") and self.peek()[0] == "op":
            op = self.next()[1]
            a = ("bin", op, a, self.unary())
        return a

    def unary(self):
        if self.peek()[1] in ("-", "+", "~") and self.peek()[0] == "op":
            op = self.next()[1]
            return ("un", op, self.unary())
        return self.power()

    def power(self):
        a = self.postfix()
        while self.peek()[1] in ("^", ".^") and self.peek()[0] == "op":
            op = self.next()[1]
            if self.peek()[1] in ("-", "+") and self.peek()[0] == "op":
                sign = self.next()[1]
                b = ("un", sign, self.postfix())
            else:
                b = self.postfix()
            a = ("bin", op, a, b)
        return a

    def postfix(self):
        a = self.primary()
        while True:
            tok = self.peek()
            if tok[1] == "(" and tok[0] == "op" and not (self.in_matrix and self.t[self.i - 1][2]):
                self.next()
                a = ("index", a, self.args(")"))
            elif tok[1] == "{" and tok[0] == "op" and not (self.in_matrix and self.t[self.i - 1][2]):
                self.next()
                a = ("cindex", a, self.args("}"))
            elif tok[1] in ("'", ".'") and tok[0] == "op":
                self.next()
                a = ("transpose", a)
            elif tok[1] == "." and tok[0] == "op" and self.peek(1)[0] == "id":
                self.next()
                a = ("field", a, self.next()[1])
            else:
                return a

    def args(self, close):
        out = []
        saved = self.in_matrix
        self.in_matrix = 0
        self.in_index += 1
        if not self.accept(close):
            while True:
                out.append(self.expr())
                if self.accept(close):
                    break
                self.expect(",")
        self.in_index -= 1
        self.in_matrix = saved
        return out

    def primary(self):
        tok = self.next()
        kind, text = tok[0], tok[1]
        if kind == "num":
            return ("num", float(text))
        if kind == "str":
            return ("str", text)
        if kind == "id":
            return ("id", text)
        if kind == "kw" and text == "end" and self.in_index:
            return ("endval",)
        if text == "(":
            saved = self.in_matrix
            self.in_matrix = 0
            e = self.expr()
            self.in_matrix = saved
            self.expect(")")
            return ("paren", e)
        if text in ("[", "{"):
            close = "]" if text == "[" else "}"
            rows, row = [], []
            self.in_matrix += 1
            saved_index = self.in_index
            self.in_index = 0
            while True:
                if self.accept(close):
                    break
                if self.accept(";"):
                    rows.append(row)
                    row = []
                    continue
                if self.accept(","):
                    continue
                row.append(self.expr())
            rows.append(row)
            self.in_matrix -= 1
            self.in_index = saved_index
            return ("matrix" if text == "[" else "cell", [r for r in rows if r])
        raise SyntaxError(f"unexpected token {text!r}")


# ---------------------------------------------------------------------------
# evaluator

class Return(Exception):
    pass


class Break(Exception):
    pass


class Continue(Exception):
    pass


class Interpreter:
    def __init__(self, paths, patches=None):
        """paths: directories searched for function files; patches:
        {function name: [(old, new), ...]} applied to a file's source before
        parsing (documented source fixes, e.g. the reference's undefined U_r)."""
        self.paths = list(paths)
        self.patches = patches or {}
        self.funcs = {}
        self.files = {}               # save/load store: name -> {var: value}

    # -- function lookup
    def function(self, name):
        if name in self.funcs:
            return self.funcs[name]
        for d in self.paths:
            p = os.path.join(d, name + ".m")
            if os.path.exists(p):
                src = open(p).read()
                for old, new in self.patches.get(name, []):
                    if old not in src:
                        raise ValueError(f"patch for {name} does not apply: {old!r}")
                    src = src.replace(old, new)
                for fname, f in Parser(lex(src)).file().items():
                    self.funcs.setdefault(fname, f)
                return self.funcs[name]
        return None

    def call(self, name, args, nout=1):
        if name in BUILTINS:
            return BUILTINS[name](self, args, nout)
        f = self.function(name)
        if f is None:
            raise NameError(f"undefined function or variable {name!r}")
        _, _, params, outs, body = f
        if len(args) > len(params):
            raise TypeError(f"{name}: too many arguments")
        env = dict(zip(params, args))
        env["__nargin__"] = len(args)
        try:
            self.block(body, env)
        except Return:
            pass
        res = []
        for o in outs[:max(nout, 1)]:
            if o not in env:
                if len(res) < nout:
                    raise NameError(f"{name}: output {o} not set")
                break
            res.append(env[o])
        return res

    # -- statements
    def block(self, stmts, env):
        for s in stmts:
            self.stmt(s, env)

    def stmt(self, s, env):
        k = s[0]
        if k == "assign":
            self.assign(s[1], self.value(s[2], env), env)
        elif k == "massign":
            targets = s[1]
            e = s[2]
            if e[0] == "index" and e[1][0] == "id" and e[1][1] not in env:
                vals = self.call(e[1][1], [self.value(a, env) for a in e[2]], len(targets))
            elif e[0] == "id" and e[0] not in env:
                vals = self.call(e[1], [], len(targets))
            else:
                raise SyntaxError("multiple assignment needs a function call")
            for t, v in zip(targets, vals):
                if not (t[0] == "un" and t[1] == "~"):
                    self.assign(t, v, env)
        elif k == "expr":
            e = s[1]
            if e[0] == "index" and e[1][0] == "id" and e[1][1] in ENV_BUILTINS and e[1][1] not in env:
                ENV_BUILTINS[e[1][1]](self, [self.value(x, env) for x in e[2]], 0, env=env)
            elif e[0] == "id" and e[1] not in env:
                self.call(e[1], [], 0)
            elif e[0] == "index" and e[1][0] == "id" and e[1][1] not in env:
                self.call(e[1][1], [self.value(a, env) for a in e[2]], 0)
            else:
                self.value(e, env)
        elif k == "for":
            rng = num(self.value(s[2], env))
            for col in range(rng.shape[1]):
                env[s[1]] = rng[:, col:col + 1].copy()
                try:
                    self.block(s[3], env)
                except Break:
                    break
                except Continue:
                    continue
        elif k == "while":
            while truth(self.value(s[1], env)):
                try:
                    self.block(s[2], env)
                except Break:
                    break
                except Continue:
                    continue
        elif k == "if":
            for cond, body in s[1]:
                if truth(self.value(cond, env)):
                    self.block(body, env)
                    return
            self.block(s[2], env)
        elif k == "switch":
            subject = self.value(s[1], env)
            for label, body in s[2]:
                lv = self.value(label, env)
                options = lv.items if isinstance(lv, Cell) else [lv]
                if any(_case_match(subject, o) for o in options):
                    self.block(body, env)
                    return
            self.block(s[3], env)
        elif k == "return":
            raise Return()
        elif k == "break":
            raise Break()
        elif k == "continue":
            raise Continue()
        else:
            raise SyntaxError(f"statement {k}")

    # -- indexing helpers
    def subscripts(self, args, env, shape):
        nd = len(args)
        subs = []
        for d, a in enumerate(args):
            if a[0] == "colon":
                subs.append(slice(None))
                continue
            if nd == 1:
                endv = shape[0] * shape[1]
            else:
                endv = shape[d] if d < 2 else 1
            env["__end__"] = endv
            v = num(self.value(a, env))
            if v.dtype == bool:
                idx = np.flatnonzero(v.ravel(order="F"))
            else:
                idx = v.ravel(order="F").astype(np.int64) - 1
                if np.any(idx < 0):
                    raise IndexError("index must be positive")
            subs.append(idx)
        return subs

    def index(self, base, args, env):
        if isinstance(base, str):
            base = num(base)
        if sp.issparse(base):
            base = base.toarray()
        a = num(base)
        subs = self.subscripts(args, env, a.shape)
        if len(subs) == 1:
            flat = a.ravel(order="F")
            s = subs[0]
            if isinstance(s, slice):
                return flat.reshape(-1, 1).copy()
            out = flat[s]
            iv = args[0]
            # a vector indexed by a vector keeps the orientation of the source
            if a.shape[0] == 1:
                return out.reshape(1, -1)
            return out.reshape(-1, 1)
        r, c = subs[0], subs[1]
        if isinstance(r, slice):
            r = np.arange(a.shape[0])
        if isinstance(c, slice):
            c = np.arange(a.shape[1])
        return a[np.ix_(r, c)].copy()

    def assign(self, target, val, env):
        if target[0] == "id":
            env[target[1]] = val
            return
        if target[0] == "cindex":
            name = target[1][1]
            cell = env.get(name)
            if not isinstance(cell, Cell):
                cell = Cell()
            k = int(scalar(self.value(target[2][0], env))) - 1
            while len(cell.items) <= k:
                cell.items.append(np.zeros((0, 0)))
            cell.items[k] = val
            if cell.shape[0] <= 1:
                cell.shape = (1, len(cell.items))
            env[name] = cell
            return
        if target[0] != "index" or target[1][0] != "id":
            raise SyntaxError("unsupported assignment target")
        name = target[1][1]
        cur = env.get(name)
        a = np.zeros((0, 0)) if cur is None else num(cur)
        a = np.array(a, dtype=float, order="F")
        v = num(val)
        subs = self.subscripts(target[2], env, a.shape)
        if len(subs) == 1:
            flat = a.ravel(order="F").copy()
            s = subs[0]
            idx = np.arange(flat.size) if isinstance(s, slice) else s
            need = int(idx.max()) + 1 if idx.size else 0
            if need > flat.size:
                if a.shape[0] <= 1:
                    flat = np.concatenate([flat, np.zeros(need - flat.size)])
                    newshape = (1, need)
                else:
                    raise IndexError("linear growth of a matrix")
            else:
                newshape = a.shape
            flat[idx] = v.ravel(order="F") if v.size != 1 else v.flat[0]
            env[name] = flat.reshape(newshape, order="F")
            return
        r, c = subs[0], subs[1]
        rows = np.arange(a.shape[0]) if isinstance(r, slice) else r
        cols = np.arange(a.shape[1]) if isinstance(c, slice) else c
        if isinstance(r, slice) and a.shape[0] == 0:
            rows = np.arange(v.shape[0])
        nr = max(a.shape[0], int(rows.max()) + 1 if rows.size else 0)
        nc = max(a.shape[1], int(cols.max()) + 1 if cols.size else 0)
        if (nr, nc) != a.shape:
            g = np.zeros((nr, nc), order="F")
            g[:a.shape[0], :a.shape[1]] = a
            a = g
        if v.size == 1:
            a[np.ix_(rows, cols)] = v.flat[0]
        else:
            a[np.ix_(rows, cols)] = v.reshape(len(rows), len(cols), order="F")
        env[name] = a

    # -- expressions
    def value(self, e, env):
        k = e[0]
        if k == "num":
            return np.array([[e[1]]])
        if k == "str":
            return e[1]
        if k == "id":
            name = e[1]
            if name in env:
                return env[name]
            if name == "nargin":
                return np.array([[float(env.get("__nargin__", 0))]])
            r = self.call(name, [], 1)
            return r[0] if r else None
        if k == "endval":
            return np.array([[float(env["__end__"])]])
        if k == "paren":
            return self.value(e[1], env)
        if k == "index":
            b = e[1]
            if b[0] == "id" and b[1] not in env:
                r = self.call(b[1], [self.value(a, env) for a in e[2]], 1)
                return r[0] if r else None
            base = self.value(b, env)
            saved = env.get("__end__")
            out = self.index(base, e[2], env)
            env["__end__"] = saved
            return out
        if k == "cindex":
            c = self.value(e[1], env)
            if not isinstance(c, Cell):
                raise TypeError("brace indexing of a non-cell")
            sub = [int(scalar(self.value(a, env))) - 1 for a in e[2]]
            kidx = sub[0] if len(sub) == 1 else sub[0] + sub[1] * c.shape[0]
            return c.items[kidx]
        if k == "field":
            return self.value(e[1], env)[e[2]]
        if k == "transpose":
            v = self.value(e[1], env)
            return v.T.copy() if not isinstance(v, str) else num(v).T
        if k == "range":
            a = scalar(self.value(e[1], env))
            s = 1.0 if e[2] is None else scalar(self.value(e[2], env))
            b = scalar(self.value(e[3], env))
            return colon(a, s, b)
        if k == "un":
            v = self.value(e[2], env)
            if e[1] == "-":
                return -num(v)
            if e[1] == "+":
                return num(v)
            return ~(num(v) != 0)
        if k == "||":
            return np.array([[truth(self.value(e[1], env)) or truth(self.value(e[2], env))]])
        if k == "&&":
            return np.array([[truth(self.value(e[1], env)) and truth(self.value(e[2], env))]])
        if k == "bin":
            return binop(e[1], self.value(e[2], env), self.value(e[3], env))
        if k == "matrix":
            if not e[1]:
                return np.zeros((0, 0))
            cells = [[self.value(x, env) for x in r] for r in e[1]]
            if any(isinstance(v, Cell) for r in cells for v in r):
                # concatenation of cell rows of equal width: [a ; b] -> 2 x n cell
                rows_ = [sum((v.items for v in r), []) for r in cells]
                ncol = len(rows_[0])
                items = [rows_[i][j] for j in range(ncol) for i in range(len(rows_))]
                return Cell(items, (len(rows_), ncol))
            rows = []
            for r in e[1]:
                vals = [self.value(x, env) for x in r]
                if all(isinstance(v, str) for v in vals):
                    rows.append("".join(vals))
                    continue
                parts = [num(v) for v in vals if not (isinstance(v, np.ndarray) and v.size == 0)]
                rows.append(np.hstack(parts) if parts else np.zeros((0, 0)))
            if len(rows) == 1:
                return rows[0]
            parts = [num(r) for r in rows if num(r).size]
            return np.vstack(parts) if parts else np.zeros((0, 0))
        if k == "cell":
            return Cell([self.value(x, env) for r in e[1] for x in r])
        raise SyntaxError(f"expression {k}")


def colon(a, s, b):
    if s == 0 or (s > 0 and a > b) or (s < 0 and a < b):
        return np.zeros((1, 0))
    n = int(math.floor((b - a) / s * (1 + 1e-15) + 1e-10)) + 1
    k = np.arange(n, dtype=float)
    out = a + k * s
    # as MATLAB's colon: the second half counted back from the last element
    last = a + (n - 1) * s
    half = n // 2
    out[half:] = last - (n - 1 - np.arange(half, n)) * s
    return out.reshape(1, -1)


def binop(op, x, y):
    if op == "*" and (sp.issparse(x) or sp.issparse(y)):
        if sp.issparse(x) and not sp.issparse(y):
            yy = num(y)
            if yy.size == 1:
                return x.multiply(yy.flat[0]).toarray()
            return np.asarray(x @ yy)
        if sp.issparse(y) and not sp.issparse(x):
            xx = num(x)
            if xx.size == 1:
                return y.multiply(xx.flat[0]).toarray()
            return np.asarray(xx @ y)
    a, b = num(x), num(y)
    if op == "+":
        return a + b
    if op == "-":
        return a - b
    if op == ".*":
        return a * b
    if op == "./":
        with np.errstate(divide="ignore", invalid="ignore"):
            return a / b
    if op == ".^":
        return np.power(a, b)
    if op == "*":
        if a.size == 1 or b.size == 1:
            return a * b
        return a @ b
    if op == "/":
        if b.size == 1:
            with np.errstate(divide="ignore", invalid="ignore"):
                return a / b
        raise NotImplementedError("matrix right division")
    if op == "^":
        if a.size == 1 and b.size == 1:
            return np.power(a, b)
        raise NotImplementedError("matrix power")
    if op == "==":
        return a == b
    if op == "~=":
        return a != b
    if op == "<":
        return a < b
    if op == "<=":
        return a <= b
    if op == ">":
        return a > b
    if op == ">=":
        return a >= b
    if op == "&":
        return (a != 0) & (b != 0)
    if op == "|":
        return (a != 0) | (b != 0)
    raise NotImplementedError(op)


# ---------------------------------------------------------------------------
# builtins: f(interp, args, nout) -> list of outputs

def _size(it, a, nout):
    v = a[0]
    shape = (1, len(v)) if isinstance(v, str) else (v.shape if sp.issparse(v) else num(v).shape)
    if len(a) > 1:
        return [np.array([[float(shape[int(scalar(a[1])) - 1])]])]
    if nout <= 1:
        return [np.array([[float(shape[0]), float(shape[1])]])]
    return [np.array([[float(s)]]) for s in shape][:nout]


def _zeros(it, a, nout):
    if len(a) == 1 and num(a[0]).size == 2:
        a = [num(a[0]).flat[0], num(a[0]).flat[1]]
    dims = [int(scalar(x)) for x in a] or [1]
    if len(dims) == 1:
        dims = dims * 2
    return [np.zeros(tuple(dims), order="F")]


def _ones(it, a, nout):
    return [np.ones(_zeros(it, a, nout)[0].shape, order="F")]


def _reshape(it, a, nout):
    v = num(a[0])
    m, n = int(scalar(a[1])), int(scalar(a[2]))
    return [v.ravel(order="F").reshape((m, n), order="F")]


def _minmax(fn):
    def f(it, a, nout):
        v = num(a[0])
        if len(a) >= 2 and num(a[1]).size:
            return [fn(v, num(a[1]))]
        if v.shape[0] == 1 or v.shape[1] == 1:
            return [np.array([[fn.reduce(v.ravel())]])]
        return [fn.reduce(v, axis=0).reshape(1, -1)]
    return f


def _sparse(it, a, nout):
    if len(a) == 1:
        return [sp.csc_matrix(num(a[0]))]
    I = num(a[0]).ravel(order="F").astype(np.int64) - 1
    J = num(a[1]).ravel(order="F").astype(np.int64) - 1
    V = num(a[2]).ravel(order="F")
    m, n = int(scalar(a[3])), int(scalar(a[4]))
    return [sp.csc_matrix(sp.coo_matrix((V, (I, J)), shape=(m, n)))]


def _repmat(it, a, nout):
    return [np.tile(num(a[0]), (int(scalar(a[1])), int(scalar(a[2]))))]


def _num2str(it, a, nout):
    v = scalar(a[0])
    return [str(int(v)) if float(v).is_integer() else repr(float(v))]


def _norm_name(name):
    return name[:-4] if name.endswith(".mat") else name


BUILTINS = {
    "size": _size,
    "zeros": _zeros,
    "ones": _ones,
    "reshape": _reshape,
    "floor": lambda it, a, n: [np.floor(num(a[0]))],
    "ceil": lambda it, a, n: [np.ceil(num(a[0]))],
    "round": lambda it, a, n: [np.sign(num(a[0])) * np.floor(np.abs(num(a[0])) + 0.5)],
    "abs": lambda it, a, n: [np.abs(num(a[0]))],
    "sqrt": lambda it, a, n: [np.sqrt(num(a[0]))],
    "log": lambda it, a, n: [np.log(num(a[0]))],
    "exp": lambda it, a, n: [np.exp(num(a[0]))],
    "max": _minmax(np.maximum),
    "min": _minmax(np.minimum),
    "length": lambda it, a, n: [np.array([[float(max(num(a[0]).shape) if num(a[0]).size else 0)]])],
    "numel": lambda it, a, n: [np.array([[float(num(a[0]).size)]])],
    "isempty": lambda it, a, n: [np.array([[a[0] is None or (not isinstance(a[0], Cell) and num(a[0]).size == 0)]])],
    "rem": lambda it, a, n: [np.fmod(num(a[0]), num(a[1]))],
    "mod": lambda it, a, n: [num(a[0]) - np.floor(num(a[0]) / num(a[1])) * num(a[1])],
    "sparse": _sparse,
    "full": lambda it, a, n: [num(a[0])],
    "repmat": _repmat,
    "num2str": _num2str,
    "imagesc": lambda it, a, n: [],
    "drawnow": lambda it, a, n: [],
    "caxis": lambda it, a, n: [np.array([[0.0, 1.0]])],
    "disp": lambda it, a, n: [],
    "fprintf": lambda it, a, n: [],
    "tic": lambda it, a, n: [],
    "toc": lambda it, a, n: [np.array([[0.0]])],
    "pi": lambda it, a, n: [np.array([[math.pi]])],
    "fix": lambda it, a, n: [np.trunc(num(a[0]))],
    "lower": lambda it, a, n: [a[0].lower()],
    "cell": lambda it, a, n: [Cell([np.zeros((0, 0))] * (int(scalar(a[0])) * int(scalar(a[1]))),
                                   (int(scalar(a[0])), int(scalar(a[1]))))],
    "sum": lambda it, a, n: [np.sum(num(a[0]), axis=0, keepdims=True) if num(a[0]).shape[0] > 1
                             else np.sum(num(a[0]), axis=1, keepdims=True)],
    "find": lambda it, a, n: [(np.flatnonzero(num(a[0]).ravel(order="F")) + 1.0).reshape(-1, 1)],
    "datetime": lambda it, a, n: ["now"],
    "string": lambda it, a, n: [str(a[0])],
    "isfield": lambda it, a, n: [np.array([[isinstance(a[0], dict) and a[1] in a[0]]])],
    "error": lambda it, a, n: (_ for _ in ()).throw(MatlabError(a[0], a[1] if len(a) > 1 else "")),
}


def _install_saveload():
    """save(name, 'var', ...) / load(name) / clear(names) work on the caller's
    variables: the interpreter passes them the caller's environment."""
    def save(it, a, nout, env=None):
        name = _norm_name(a[0])
        it.files[name] = {v: env[v].copy() if isinstance(env[v], np.ndarray) else env[v] for v in a[1:]}
        return []

    def load(it, a, nout, env=None):
        name = _norm_name(a[0])
        data = it.files[name]
        if nout >= 1:
            raise NotImplementedError("load into a struct")
        env.update({k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in data.items()})
        return []
    def clear(it, a, nout, env=None):
        for name in a:
            env.pop(name, None)
        return []
    return {"save": save, "load": load, "clear": clear}


ENV_BUILTINS = _install_saveload()
