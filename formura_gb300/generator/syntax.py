"""Parser for the Formura stencil language.

Restates the grammar of ``src/Formura/Parser.hs`` (and the AST of
``src/Formura/Syntax.hs``) for the language subset that Formura programs use:

* lexical rules: identifiers ``Parser.hs:113-145``, keywords ``Parser.hs:77-85``,
  ``#`` comments and ``\\`` line continuation ``Parser.hs:88-99``; newlines and
  ``;`` delimit statements ``Parser.hs:304-307``;
* operator table ``Parser.hs:199-211`` (highest first): ``.`` (right),
  ``**``, ``* /``, prefix ``+ -``, ``+ -``, ``&&``, ``||``, comparisons
  (non-associative);
* application chains and grid indexing ``Parser.hs:249-263``; n+k patterns
  ``Parser.hs:183-191``; tuples, where one element is a parenthesised
  expression ``Parser.hs:162-172``;
* ``let``/``fun``/``if`` ``Parser.hs:270-295``;
* ``begin function ... end function`` sugar ``Parser.hs:314-346``;
* typed declarations with ``const``/``extern``/``manifest`` ``Parser.hs:349-438``;
* ``dimension``/``axes`` declarations ``Parser.hs:469-491``;
* the program: injected ``dx..`` (exact rationals) and ``total_grid_..``
  ``Parser.hs:493-511``, then grid indices padded to the dimension
  (``Desugar.hs:172-194``).

AST nodes are plain tuples whose first element names the form:
``('imm', Fraction)``, ``('ident', name)``, ``('tuple', [..])``,
``('grid', [(name, Fraction)..], expr)``, ``('vector', name, expr)``,
``('apply', f, x)``, ``('lambda', lhs, body)``, ``('let', binding, body)``,
``('uniop', op, a)``, ``('binop', op, a, b)``, ``('triop', 'ite', c, a, b)``.
A binding is a list of statements ``('subst', lhs, rhs)`` and
``('typedecl', modifiers, type, lhs)``.  Types: ``('elem', name)``,
``('gridtype', [Fraction..], type)``, ``('top',)``, ``('fun',)``,
``('tuple', [..])``.
"""
from __future__ import annotations

import re
from dataclasses import dataclass, field
from fractions import Fraction
from typing import List, Optional, Tuple

from .config import NumericalConfig


class FormuraSyntaxError(ValueError):
    pass


KEYWORDS = {"begin", "end", "function", "returns", "let", "in", "fun", "dimension",
            "axes", "grid_struct_type_name", "grid_struct_instance_name", "if", "then",
            "else", "const", "extern", "manifest",
            "+", "-", "*", "/", ".", "**", "::", "=", ",", "&&", "||",
            "<?", ">?", "<%", "<=", "==", "!=", ">=", "<", ">"}
COMPARISONS = {"<=", "==", "!=", ">=", "<", ">"}
ELEMENT_TYPES = ["void", "bool", "int", "Rational", "float", "double", "real", "Real"]

_SYMBOL_EXCLUDED = set("\"#();[\\]{}")


def _is_symbol_char(c: str) -> bool:
    return (c.isprintable() and not (c.isalnum() or c == "_" or c == "'")
            and not c.isspace() and c not in _SYMBOL_EXCLUDED)


@dataclass
class Tok:
    kind: str      # 'id', 'num', 'sym', 'punct', 'nl', 'eof'
    text: str
    line: int
    value: object = None


_NUM_RE = re.compile(r"[0-9]+(\.[0-9]+)?([eE][+-]?[0-9]+)?")


def tokenize(src: str) -> List[Tok]:
    toks: List[Tok] = []
    i, n, line = 0, len(src), 1
    while i < n:
        c = src[i]
        if c == "\n":
            toks.append(Tok("nl", "\n", line))
            line += 1
            i += 1
        elif c == "\\":
            # line continuation: '\' whitespace* newline
            j = i + 1
            while j < n and src[j] in " \t\r":
                j += 1
            if j < n and src[j] == "\n":
                line += 1
                i = j + 1
            else:
                raise FormuraSyntaxError(f"line {line}: stray backslash")
        elif c.isspace():
            i += 1
        elif c == "#":
            while i < n and src[i] != "\n":
                i += 1
        elif c.isdigit():
            m = _NUM_RE.match(src, i)
            text = m.group(0)
            toks.append(Tok("num", text, line, Fraction(text)))
            i = m.end()
        elif c.isalpha():
            j = i + 1
            while j < n and (src[j].isalnum() or src[j] in "_'"):
                j += 1
            toks.append(Tok("id", src[i:j], line))
            i = j
        elif c in "()[];":
            toks.append(Tok("punct", c, line))
            i += 1
        elif c == ",":
            toks.append(Tok("sym", ",", line))
            i += 1
        elif _is_symbol_char(c):
            j = i + 1
            while j < n and _is_symbol_char(src[j]) and src[j] != ",":
                j += 1
            toks.append(Tok("sym", src[i:j], line))
            i = j
        else:
            raise FormuraSyntaxError(f"line {line}: unexpected character {c!r}")
    toks.append(Tok("nl", "\n", line))
    toks.append(Tok("eof", "", line))
    return toks


@dataclass
class Program:
    dimension: int
    axes: List[str]
    statements: list
    grid_struct_type_name: str = "Formura_Grid_Struct"
    grid_struct_instance_name: str = "formura_data"
    nc: Optional[NumericalConfig] = None
    extent_statements: list = field(default_factory=list)

    @property
    def binding(self):
        return self.extent_statements + self.statements


class _Parser:
    def __init__(self, toks: List[Tok]):
        self.t = toks
        self.p = 0

    # -- token helpers -------------------------------------------------
    def peek(self, k=0) -> Tok:
        return self.t[self.p + k]

    def err(self, msg):
        tk = self.peek()
        raise FormuraSyntaxError(f"line {tk.line}: {msg} (at {tk.text!r})")

    def is_sym(self, s, k=0):
        tk = self.peek(k)
        return tk.kind == "sym" and tk.text == s

    def is_punct(self, s, k=0):
        tk = self.peek(k)
        return tk.kind == "punct" and tk.text == s

    def is_kw(self, s, k=0):
        tk = self.peek(k)
        return tk.kind == "id" and tk.text == s

    def expect_sym(self, s):
        if not self.is_sym(s):
            self.err(f"expected {s!r}")
        self.p += 1

    def expect_punct(self, s):
        if not self.is_punct(s):
            self.err(f"expected {s!r}")
        self.p += 1

    def expect_kw(self, s):
        if not self.is_kw(s):
            self.err(f"expected keyword {s!r}")
        self.p += 1

    def skip_nl(self):
        while self.peek().kind == "nl" or self.is_punct(";"):
            self.p += 1

    def at_ident(self, k=0):
        tk = self.peek(k)
        return tk.kind == "id" and tk.text not in KEYWORDS

    def ident_name(self) -> str:
        if not self.at_ident():
            self.err("expected identifier")
        s = self.peek().text
        self.p += 1
        return s

    # -- program -------------------------------------------------------
    def program(self):
        decls, stmts = [], []
        self.skip_nl()
        while self.peek().kind != "eof":
            if self.peek().kind == "id" and self.peek().text in (
                    "dimension", "axes", "grid_struct_type_name", "grid_struct_instance_name"):
                decls.append(self.special_decl())
            else:
                stmts.extend(self.statement_compound())
            if self.peek().kind != "eof":
                if not (self.peek().kind == "nl" or self.is_punct(";")):
                    self.err("expected end of statement")
                self.skip_nl()
        return decls, stmts

    def special_decl(self):
        kw = self.peek().text
        self.p += 1
        self.expect_sym("::")
        if kw == "dimension":
            tk = self.peek()
            if tk.kind != "num" or not isinstance(tk.value, Fraction) or tk.value.denominator != 1:
                self.err("dimension must be a natural number")
            self.p += 1
            return ("dimension", int(tk.value))
        if kw == "axes":
            xs = [self.ident_name()]
            while self.is_sym(","):
                self.p += 1
                xs.append(self.ident_name())
            return ("axes", xs)
        return (kw, self.ident_name())

    def statement_compound(self):
        if self.is_kw("begin"):
            return self.function_sugar()
        return self.type_value_statements()

    def function_sugar(self):
        self.expect_kw("begin")
        self.expect_kw("function")
        # returns-form: f(x) returns y ; equal-form: y = f(x)
        save = self.p
        form = None
        try:
            fn = self.ident_name()
            inx = self.tuple_of(self.lexpr)
            if self.is_kw("returns"):
                self.p += 1
                outx = self.rexpr()
                form = (fn, inx, outx)
        except FormuraSyntaxError:
            form = None
        if form is None:
            self.p = save
            outx = self.rexpr()
            self.expect_sym("=")
            fn = self.ident_name()
            inx = self.tuple_of(self.lexpr)
            form = (fn, inx, outx)
        fn, inx, outx = form
        if not (self.peek().kind == "nl" or self.is_punct(";")):
            self.err("expected newline after function header")
        body = self.binding(until="end")
        self.expect_kw("end")
        self.expect_kw("function")
        return [("subst", ("ident", fn), ("lambda", inx, ("let", body, outx)))]

    def binding(self, until):
        stmts = []
        self.skip_nl()
        while not self.is_kw(until):
            if self.peek().kind == "eof":
                self.err(f"missing '{until}'")
            stmts.extend(self.statement_compound())
            if not (self.peek().kind == "nl" or self.is_punct(";") or self.is_kw(until)):
                self.err("expected end of statement")
            self.skip_nl()
        return stmts

    def _has_type_prefix(self) -> bool:
        j = self.p
        depth = 0
        while True:
            tk = self.t[j]
            if tk.kind in ("eof",) or (tk.kind == "nl" and depth == 0) or (
                    tk.kind == "punct" and tk.text == ";" and depth == 0):
                return False
            if tk.kind == "punct" and tk.text in "([":
                depth += 1
            elif tk.kind == "punct" and tk.text in ")]":
                depth -= 1
            elif tk.kind == "sym" and tk.text == "::" and depth == 0:
                return True
            elif tk.kind == "sym" and tk.text == "=" and depth == 0:
                return False
            j += 1

    def type_value_statements(self):
        if self._has_type_prefix():
            mods, typ = self.mod_type_expr()
            self.expect_sym("::")
            items = []
            while True:
                lhs = self.lexpr()
                rhs = None
                if self.is_sym("="):
                    self.p += 1
                    rhs = self.rexpr()
                items.append((lhs, rhs))
                if self.is_sym(","):
                    self.p += 1
                    continue
                break
            out = [("typedecl", mods, typ, lhs) for lhs, _ in items]
            out += [("subst", lhs, rhs) for lhs, rhs in items if rhs is not None]
            return out
        lhs = self.lexpr()
        self.expect_sym("=")
        rhs = self.rexpr()
        return [("subst", lhs, rhs)]

    def mod_type_expr(self):
        mods = []
        while self.peek().kind == "id" and self.peek().text in ("const", "extern", "manifest"):
            mods.append(self.peek().text)
            self.p += 1
        typ = ("top",)
        if not self.is_sym("::") and not (self.peek().kind == "id" and self.peek().text in ("const", "extern", "manifest")):
            typ = self.type_fexpr()
        while self.peek().kind == "id" and self.peek().text in ("const", "extern", "manifest"):
            mods.append(self.peek().text)
            self.p += 1
        return mods, typ

    def type_fexpr(self):
        if self.is_punct("("):
            t = self.tuple_of(self.type_fexpr)
        elif self.is_kw("function"):
            self.p += 1
            t = ("fun",)
        elif self.peek().kind == "id" and self.peek().text in ELEMENT_TYPES:
            t = ("elem", self.peek().text)
            self.p += 1
        else:
            self.err("expected a type")
        while self.is_punct("["):
            self.p += 1
            offs = []
            if not self.is_punct("]"):
                offs.append(self.const_rational())
                while self.is_sym(","):
                    self.p += 1
                    offs.append(self.const_rational())
            self.expect_punct("]")
            t = ("gridtype", offs, t)
        return t

    # -- l-expressions -------------------------------------------------
    def lexpr(self):
        if self.is_punct("("):
            f = self.tuple_of(self.lexpr)
        else:
            f = ("ident", self.ident_name())
        while True:
            if self.is_punct("["):
                f = ("grid", self.grid_indices(), f)
            elif self.is_punct("(") and self.at_ident(1) and self.is_punct(")", 2):
                self.p += 1
                name = self.ident_name()
                self.p += 1
                f = ("vector", name, f)
            else:
                return f

    def grid_indices(self):
        self.expect_punct("[")
        out = []
        if not self.is_punct("]"):
            out.append(self.n_plus_k())
            while self.is_sym(","):
                self.p += 1
                out.append(self.n_plus_k())
        self.expect_punct("]")
        return out

    def n_plus_k(self):
        name = ""
        if self.at_ident():
            name = self.ident_name()
        k = Fraction(0)
        if self.is_sym("+") or self.is_sym("-"):
            sign = self.peek().text
            self.p += 1
            k = self.const_rational()
            if sign == "-":
                k = -k
        if not (self.is_sym(",") or self.is_punct("]")):
            self.err("malformed n+k index")
        return (name, k)

    def const_rational(self) -> Fraction:
        e = self.rexpr_over(self.imm_only)
        return _eval_const(e)

    def imm_only(self):
        tk = self.peek()
        if tk.kind == "num":
            self.p += 1
            return ("imm", tk.value)
        if self.is_punct("("):
            return self.tuple_of(lambda: self.rexpr_over(self.imm_only))
        self.err("expected a constant")

    # -- r-expressions -------------------------------------------------
    def tuple_of(self, p):
        self.expect_punct("(")
        xs = []
        if not self.is_punct(")"):
            xs.append(p())
            while self.is_sym(","):
                self.p += 1
                xs.append(p())
        self.expect_punct(")")
        if len(xs) == 1:
            return xs[0]
        return ("tuple", xs)

    def rexpr(self):
        return self.rexpr_over(self.fexpr)

    def rexpr_over(self, term):
        # comparisons: lowest, non-associative
        a = self._or(term)
        if self.peek().kind == "sym" and self.peek().text in COMPARISONS:
            op = self.peek().text
            self.p += 1
            b = self._or(term)
            if self.peek().kind == "sym" and self.peek().text in COMPARISONS:
                self.err("comparison operators are non-associative")
            return ("binop", op, a, b)
        return a

    def _or(self, term):
        a = self._and(term)
        while self.is_sym("||"):
            self.p += 1
            a = ("binop", "||", a, self._and(term))
        return a

    def _and(self, term):
        a = self._add(term)
        while self.is_sym("&&"):
            self.p += 1
            a = ("binop", "&&", a, self._add(term))
        return a

    def _add(self, term):
        a = self._unary(term)
        while self.is_sym("+") or self.is_sym("-"):
            op = self.peek().text
            self.p += 1
            a = ("binop", op, a, self._unary(term))
        return a

    def _unary(self, term):
        if self.is_sym("+") or self.is_sym("-"):
            op = self.peek().text
            self.p += 1
            return ("uniop", op, self._mul(term))
        return self._mul(term)

    def _mul(self, term):
        a = self._pow(term)
        while self.is_sym("*") or self.is_sym("/"):
            op = self.peek().text
            self.p += 1
            a = ("binop", op, a, self._pow(term))
        return a

    def _pow(self, term):
        a = self._dot(term)
        while self.is_sym("**"):
            self.p += 1
            a = ("binop", "**", a, self._dot(term))
        return a

    def _dot(self, term):
        a = term()
        if self.is_sym("."):
            self.p += 1
            return ("binop", ".", a, self._dot(term))
        return a

    def _starts_aexpr(self):
        tk = self.peek()
        if tk.kind == "num":
            return True
        if tk.kind == "punct" and tk.text == "(":
            return True
        if tk.kind == "id":
            return tk.text in ("let", "fun", "if") or tk.text not in KEYWORDS
        return False

    def fexpr(self):
        f = self.aexpr()
        while True:
            if self.is_punct("["):
                f = ("grid", self.grid_indices(), f)
            elif self._starts_aexpr():
                f = ("apply", f, self.aexpr())
            else:
                return f

    def aexpr(self):
        tk = self.peek()
        if tk.kind == "punct" and tk.text == "(":
            return self.tuple_of(self.rexpr)
        if tk.kind == "id" and tk.text == "let":
            self.p += 1
            b = self.binding(until="in")
            self.expect_kw("in")
            return ("let", b, self.rexpr())
        if tk.kind == "id" and tk.text == "fun":
            self.p += 1
            lhs = self.tuple_of(self.lexpr)
            return ("lambda", lhs, self.rexpr())
        if tk.kind == "id" and tk.text == "if":
            self.p += 1
            c = self.rexpr()
            self.expect_kw("then")
            a = self.rexpr()
            self.expect_kw("else")
            b = self.rexpr()
            return ("triop", "ite", c, a, b)
        if tk.kind == "num":
            self.p += 1
            return ("imm", tk.value)
        if self.at_ident():
            self.p += 1
            return ("ident", tk.text)
        self.err("expected an expression")


def _eval_const(e) -> Fraction:
    """``evalCRE`` (``Parser.hs:449-457``)."""
    k = e[0]
    if k == "imm":
        return e[1]
    if k == "uniop":
        v = _eval_const(e[2])
        return v if e[1] == "+" else -v
    if k == "binop" and e[1] in "+-*/":
        a, b = _eval_const(e[2]), _eval_const(e[3])
        return {"+": a + b, "-": a - b, "*": a * b, "/": a / b}[e[1]]
    raise FormuraSyntaxError("unsupported operator in const rational expression")


def _pad_grids(node, dim):
    """``desugar`` (``Desugar.hs:172-194``): pad grid indices/offsets to ``dim``."""
    if isinstance(node, tuple):
        if not node:
            return node
        k = node[0]
        if k == "grid":
            idx = list(node[1])[:dim] + [("", Fraction(0))] * max(0, dim - len(node[1]))
            return ("grid", idx, _pad_grids(node[2], dim))
        if k == "gridtype":
            offs = list(node[1])[:dim] + [Fraction(0)] * max(0, dim - len(node[1]))
            return ("gridtype", offs, _pad_grids(node[2], dim))
        return tuple(_pad_grids(x, dim) for x in node)
    if isinstance(node, list):
        return [_pad_grids(x, dim) for x in node]
    return node


def parse_program(src: str, nc: NumericalConfig) -> Program:
    """``program`` (``Parser.hs:493-511``) followed by ``desugar``."""
    p = _Parser(tokenize(src))
    decls, stmts = p.program()
    dims = [v for k, v in decls if k == "dimension"]
    if len(dims) != 1:
        raise FormuraSyntaxError("no dimension declaration found." if not dims
                                 else "multiple dimension declaration found.")
    dim = dims[0]
    axes_l = [v for k, v in decls if k == "axes"]
    if len(axes_l) != 1:
        raise FormuraSyntaxError("no axes declaration found." if not axes_l
                                 else "multiple axes declaration found.")
    axes = axes_l[0]
    if len(axes) != dim:
        raise FormuraSyntaxError("number of declared axes does not match the declared dimension.")
    prog = Program(dimension=dim, axes=axes, statements=_pad_grids(stmts, dim), nc=nc)
    for k, v in decls:
        if k == "grid_struct_type_name" and v:
            prog.grid_struct_type_name = v
        if k == "grid_struct_instance_name" and v:
            prog.grid_struct_instance_name = v
    if len(nc.length_per_node) < dim or len(nc.grid_per_node) < dim:
        raise FormuraSyntaxError("numerical config has fewer axes than the program")
    mpi = nc.mpi_shape if nc.mpi_shape is not None else [1] * dim
    ext = []
    for a, l, n in zip(axes, nc.length_per_node, nc.grid_per_node):
        ext.append(("subst", ("ident", "d" + a), ("imm", Fraction(l) / n)))
    for a, n, m in zip(axes, nc.grid_per_node, mpi):
        ext.append(("subst", ("ident", "total_grid_" + a), ("imm", Fraction(n * m))))
    prog.extent_statements = ext
    return prog
