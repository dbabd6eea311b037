#!/usr/bin/env python3
"""Mechanical Fortran-to-C transliteration of the reference's library sources.

TEST INFRASTRUCTURE ONLY. The reference (Gturbo: Fortran 90 + OpenACC + cuFFT) cannot be compiled
here: no Fortran compiler exists in this container or on the GPU host. This script turns the
reference's own source files -- the SRCFILES list of its Makefile (Makefile:12-15), everything but
the main program -- into one C file, statement by statement, so that the reference's arithmetic
can be run on the CPU and used to pin the oracle and the golden vectors. Output goes to
``oracle/_ref/`` only (git-ignored); nothing under ``/root/reference`` is copied into the
repository.

What the transliteration keeps from the Fortran, mechanically:
  * every module variable becomes a C global ``f_<name>`` (arrays flattened, column-major, lower
    bound 1), every procedure a C function ``f_<name>`` whose arguments are passed by reference;
  * expressions keep Fortran's precedence, left-to-right association and type promotion
    (integer < real(4) < real(8) < complex(8)); ``x**n`` with an integer literal n is the product
    of n factors, ``x**y`` with a real y is ``pow``; literals keep their kind (``2.0`` is a
    real(4), ``2.0d0`` a real(8));
  * integer arithmetic wraps modulo 2^32 (the C is compiled with -fwrapv), as the LCG of
    forcing.f90:40-51 relies on;
  * array statements and sections become loop nests in array-element order;
  * ``!$acc parallel loop`` / ``!$acc kernels`` regions become ``#pragma omp parallel for`` where
    every iteration writes its own elements (the meaning of the reference's host-core build,
    ``-acc=multicore``); loops that accumulate into shared scalars or indirectly indexed arrays
    (the shell histograms of diagnostics.f90, the serial forcing loop) stay serial;
  * list-directed and unformatted reads/writes go to a small runtime (f2c_rt.c) that keeps the
    files' formats; formatted writes to the diagnostics units are captured in memory (the values
    written, and the FP64 operand of a top-level ``real()`` conversion).
What it replaces: the cuFFT calls of fft_dir.f90:12 and fft_inv.f90:12 resolve to
``cufft_shim.c``, which follows the DFT definitions cuFFT documents for D2Z/Z2D; the CUDA call
of show_mem (trunc.f90) resolves to a stub. Grid sizes are compile-time parameters, as in the
reference (modules.f90:4): ``-DF2C_NX=.. -DF2C_NY=..`` overrides any integer parameter.

Usage: python oracle/f2c_ref.py [--src DIR] [--out FILE]
"""
from __future__ import annotations

import argparse
import os
import re
import sys

DEFAULT_SRC = "/root/reference/src"
# Makefile:12-15 SRCFILES (the library part of the reference; main.f90 is the program)
REF_FILES = ["modules.f90", "defk.f90", "iniforcing.f90", "trunc.f90", "nlt.f90", "produ.f90",
             "diagnostics.f90", "rkstep.f90", "forcing.f90", "read.f90", "write.f90",
             "inieuler.f90", "fft_inv.f90", "fft_dir.f90"]

# External (non-Fortran) functions the sources call, with their C argument passing:
# 'v' = by value, 'p' = by pointer (the cufft / cudafor module interfaces).
EXTERNALS = {
    "cufftexecd2z": ("int", "vpp"),
    "cufftexecz2d": ("int", "vpp"),
    "cudamemgetinfo": ("int", "pp"),
}

ORDER = ["l", "i4", "i8", "r4", "r8", "c8"]
CTYPE = {"i4": "int", "i8": "long long", "r4": "float", "r8": "double", "c8": "double _Complex",
         "l": "int", "ch": "char"}


class F2CError(Exception):
    pass


# ----------------------------------------------------------------------------------------------
# lexing
# ----------------------------------------------------------------------------------------------
_DOTOPS = r"(?:eq|ne|lt|le|gt|ge|and|or|not|true|false|eqv|neqv)"
TOKEN_RE = re.compile(r"""
  (?P<ws>\s+)
 |(?P<boz>'[0-9a-fA-F]+'[xX])
 |(?P<str>'(?:[^']|'')*'|"(?:[^"]|"")*")
 |(?P<num>(?:\d+\.(?!""" + _DOTOPS + r"""\.)\d*|\.\d+|\d+)(?:[eEdD][+-]?\d+)?)
 |(?P<dotop>\.""" + _DOTOPS + r"""\.)
 |(?P<name>[A-Za-z_][A-Za-z_0-9]*)
 |(?P<op>\*\*|==|/=|<=|>=|::|[-+*/(),:<>=%])
""", re.X | re.I)


class Tok:
    __slots__ = ("kind", "text")

    def __init__(self, kind, text):
        self.kind, self.text = kind, text

    def __repr__(self):
        return f"{self.kind}:{self.text}"


def tokenize(s: str) -> list[Tok]:
    out, pos = [], 0
    while pos < len(s):
        m = TOKEN_RE.match(s, pos)
        if not m:
            raise F2CError(f"cannot tokenize: {s[pos:]!r} in {s!r}")
        pos = m.end()
        k = m.lastgroup
        t = m.group(k)
        if k == "ws":
            continue
        if k in ("name", "dotop"):
            t = t.lower()
        out.append(Tok(k, t))
    return out


def strip_comment(line: str) -> tuple[str, str | None]:
    """(code, directive): the code before a '!' outside quotes; an '!$acc' line's directive."""
    s = line.strip()
    if s.lower().startswith("!$acc"):
        return "", s[5:].strip().lower()
    q = None
    for i, ch in enumerate(line):
        if q:
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
        elif ch == "!":
            return line[:i], None
    return line, None


def logical_lines(text: str):
    """(label, tokens, directive) per statement; '&' continuations joined."""
    pending = ""
    for raw in text.splitlines():
        code, directive = strip_comment(raw)
        if directive is not None:
            yield None, None, directive
            continue
        code = code.rstrip()
        if code.endswith("&"):
            pending += code[:-1] + " "
            continue
        code = pending + code
        pending = ""
        if not code.strip():
            continue
        m = re.match(r"\s*(\d+)\s+(.*)$", code)
        label = None
        if m:
            label, code = int(m.group(1)), m.group(2)
        yield label, tokenize(code), None


# ----------------------------------------------------------------------------------------------
# expressions
# ----------------------------------------------------------------------------------------------
class Num:
    def __init__(self, text, t):
        self.text, self.t = text, t


class Str:
    def __init__(self, text):
        self.text = text


class Name:
    def __init__(self, name):
        self.name = name


class Ref:  # name(args): array element/section, intrinsic or function call
    def __init__(self, name, args):
        self.name, self.args = name, args


class Slice:  # lo:hi inside a subscript list (either may be None)
    def __init__(self, lo, hi):
        self.lo, self.hi = lo, hi


class Bin:
    def __init__(self, op, a, b):
        self.op, self.a, self.b = op, a, b


class Un:
    def __init__(self, op, a):
        self.op, self.a = op, a


class Cplx:
    def __init__(self, re_, im):
        self.re, self.im = re_, im


class Star:  # '*' as a format / unit specifier
    pass


BP = {".or.": 10, ".and.": 20, ".eq.": 30, ".ne.": 30, ".lt.": 30, ".le.": 30, ".gt.": 30,
      ".ge.": 30, "==": 30, "/=": 30, "<": 30, "<=": 30, ">": 30, ">=": 30, "+": 40, "-": 40,
      "*": 50, "/": 50, "**": 60}


class Parser:
    def __init__(self, toks, pos=0):
        self.toks, self.pos = toks, pos

    def peek(self, k=0):
        i = self.pos + k
        return self.toks[i] if i < len(self.toks) else None

    def next(self):
        t = self.toks[self.pos]
        self.pos += 1
        return t

    def accept(self, text):
        t = self.peek()
        if t is not None and t.text == text:
            self.pos += 1
            return True
        return False

    def expect(self, text):
        if not self.accept(text):
            raise F2CError(f"expected {text!r} at {self.toks[self.pos:]}")

    def at_end(self):
        return self.pos >= len(self.toks)

    def expr(self, rbp=0):
        left = self.prefix()
        while True:
            t = self.peek()
            if t is None or t.text not in BP or BP[t.text] <= rbp:
                # '**' is right-associative: equal binding continues
                if not (t is not None and t.text == "**" and BP["**"] > rbp - 1 and rbp == 59):
                    break
            op = self.next().text
            if op == "**":
                right = self.expr(59)
            else:
                right = self.expr(BP[op])
            left = Bin(op, left, right)
        return left

    def prefix(self):
        t = self.next()
        if t.text in ("-", "+"):
            return Un(t.text, self.expr(45))
        if t.text == ".not.":
            return Un("!", self.expr(25))
        if t.kind == "num":
            return num_literal(t.text)
        if t.kind == "boz":
            return Num(str(int(t.text[1:-2], 16)), "i4")
        if t.kind == "str":
            return Str(t.text)
        if t.text in (".true.", ".false."):
            return Num("1" if t.text == ".true." else "0", "l")
        if t.text == "*":
            return Star()
        if t.text == "(":
            e = self.expr()
            if self.accept(","):
                im = self.expr()
                self.expect(")")
                return Cplx(e, im)
            self.expect(")")
            return e
        if t.kind == "name":
            if self.accept("("):
                return Ref(t.text, self.arglist())
            return Name(t.text)
        raise F2CError(f"unexpected token {t} in expression")

    def subscript(self):
        if self.peek().text == ":":
            self.next()
            hi = None if self.peek().text in (",", ")") else self.expr()
            return Slice(None, hi)
        e = self.expr()
        if self.accept(":"):
            hi = None if self.peek().text in (",", ")") else self.expr()
            return Slice(e, hi)
        return e

    def arglist(self):
        args = []
        if self.accept(")"):
            return args
        while True:
            # keyword argument (I/O control lists): name = expr
            if (self.peek().kind == "name" and self.peek(1) is not None and self.peek(1).text == "="):
                key = self.next().text
                self.next()
                args.append(("kw", key, self.expr()))
            else:
                args.append(self.subscript())
            if self.accept(")"):
                return args
            self.expect(",")


def num_literal(text):
    t = text.lower()
    if re.fullmatch(r"\d+", t):
        return Num(t, "i4")
    if "d" in t:
        mant, ex = t.split("d")
        if mant.endswith("."):
            mant += "0"
        if mant.startswith("."):
            mant = "0" + mant
        return Num(f"{mant}e{ex}", "r8")
    c = t
    if c.endswith("."):
        c += "0"
    if c.startswith("."):
        c = "0" + c
    return Num(c + "f", "r4")  # default real kind: real(4)


def split_top(toks, sep=","):
    """Split a token list on top-level separators."""
    out, cur, depth = [], [], 0
    for t in toks:
        if t.text == "(":
            depth += 1
        elif t.text == ")":
            depth -= 1
        if t.text == sep and depth == 0:
            out.append(cur)
            cur = []
        else:
            cur.append(t)
    if cur:
        out.append(cur)
    return out


def parse_expr(toks):
    p = Parser(toks)
    e = p.expr()
    if not p.at_end():
        raise F2CError(f"trailing tokens {p.toks[p.pos:]}")
    return e


# ----------------------------------------------------------------------------------------------
# symbols
# ----------------------------------------------------------------------------------------------
class Sym:
    def __init__(self, name, t, dims=None, scope="local", charlen=0):
        self.name, self.t, self.dims, self.scope = name, t, dims, scope
        self.param = None  # initialiser expression of a parameter
        self.charlen = charlen
        self.dummy = False
        self.is_result = False

    @property
    def cname(self):
        return "f_" + self.name + ("_res" if self.is_result else "")


def parse_typespec(toks):
    """(type, charlen, rest) from a declaration's leading tokens."""
    first = toks[0].text
    rest = toks[1:]
    charlen = 0
    if first == "double" and rest and rest[0].text == "precision":
        return "r8", 0, rest[1:]
    if first in ("real", "integer", "complex", "logical", "character"):
        kind = None
        if rest and rest[0].text == "*":
            kind = int(rest[1].text)
            rest = rest[2:]
        elif rest and rest[0].text == "(":
            depth, j = 0, 0
            for j, t in enumerate(rest):
                depth += t.text == "("
                depth -= t.text == ")"
                if depth == 0:
                    break
            inner = rest[1:j]
            rest = rest[j + 1:]
            if len(inner) == 1 and inner[0].kind == "num":
                kind = int(inner[0].text)
            elif inner and inner[0].text == "kind":
                kind = "big"
        if first == "real":
            return {None: "r4", 4: "r4", 8: "r8"}[kind], 0, rest
        if first == "integer":
            return ("i8" if kind in (8, "big") else "i4"), 0, rest
        if first == "complex":
            return {None: "c8", 8: "c8", 16: "c8"}[kind], 0, rest
        if first == "logical":
            return "l", 0, rest
        if first == "character":
            charlen = kind if isinstance(kind, int) else 1
            return "ch", charlen, rest
    raise F2CError(f"not a type: {toks}")


# ----------------------------------------------------------------------------------------------
# statements (tree)
# ----------------------------------------------------------------------------------------------
class Stmt:
    def __init__(self, kind, **kw):
        self.kind = kind
        self.label = None
        self.__dict__.update(kw)


class Unit:
    def __init__(self, kind, name, args, rtype=None):
        self.kind, self.name, self.args, self.rtype = kind, name, args, rtype
        self.syms: dict[str, Sym] = {}
        self.body: list[Stmt] = []
        self.uses: list[str] = []


class Translator:
    def __init__(self):
        self.globals: dict[str, Sym] = {}
        self.modules: dict[str, list[str]] = {}
        self.units: list[Unit] = []
        self.functions: dict[str, str] = {}  # name -> result type
        self.tmp = 0

    # ---- parsing ------------------------------------------------------------------------
    def parse_file(self, text):
        lines = list(logical_lines(text))
        i = 0
        while i < len(lines):
            label, toks, directive = lines[i]
            if toks is None:
                i += 1
                continue
            head = toks[0].text
            if head == "module":
                i = self.parse_module(lines, i)
            elif head == "subroutine" or (len(toks) > 1 and "function" in [t.text for t in toks[:4]]):
                i = self.parse_unit(lines, i)
            else:
                raise F2CError(f"unexpected top-level statement {toks}")

    def parse_module(self, lines, i):
        name = lines[i][1][1].text
        self.modules[name] = []
        i += 1
        while True:
            label, toks, directive = lines[i]
            i += 1
            if toks is None:
                continue
            words = [t.text for t in toks]
            if words[0] == "end" or words[0] == "endmodule":
                return i
            if words[0] in ("use", "implicit"):
                continue
            for s in self.parse_decl(toks, scope="global"):
                self.globals[s.name] = s
                self.modules[name].append(s.name)

    def parse_decl(self, toks, scope):
        t, charlen, rest = parse_typespec(toks)
        attrs_dims, is_param = None, False
        words = [x.text for x in rest]
        if "::" in words:
            k = words.index("::")
            attr_toks, ent_toks = rest[:k], rest[k + 1:]
            for part in split_top(attr_toks):
                if not part:
                    continue
                w = part[0].text
                if w == "parameter":
                    is_param = True
                elif w == "dimension":
                    attrs_dims = [parse_expr(d) for d in split_top(part[2:-1])]
                # intent(...) and other attributes carry no arithmetic
        else:
            ent_toks = rest
        out = []
        for ent in split_top(ent_toks):
            name = ent[0].text
            dims = attrs_dims
            init = None
            j = 1
            if j < len(ent) and ent[j].text == "(":
                depth, k = 0, j
                for k in range(j, len(ent)):
                    depth += ent[k].text == "("
                    depth -= ent[k].text == ")"
                    if depth == 0:
                        break
                dims = [parse_expr(d) for d in split_top(ent[j + 1:k])]
                j = k + 1
            if j < len(ent) and ent[j].text == "=":
                init = parse_expr(ent[j + 1:])
            s = Sym(name, t, dims, scope, charlen)
            if is_param:
                s.param = init
            out.append(s)
        return out

    def parse_unit(self, lines, i):
        toks = lines[i][1]
        words = [t.text for t in toks]
        if words[0] == "subroutine":
            kind, name, rtype, k = "sub", words[1], None, 2
        else:
            fi = words.index("function")
            rtype = parse_typespec(toks[:fi])[0] if fi > 0 else "r4"
            kind, name, k = "fun", words[fi + 1], fi + 2
        args = []
        if k < len(toks) and toks[k].text == "(":
            args = [t.text for t in toks[k + 1:-1] if t.text != ","]
        u = Unit(kind, name, args, rtype)
        if kind == "fun":
            self.functions[name] = rtype
            r = Sym(name, rtype)
            r.is_result = True
            u.syms[name] = r
        i += 1
        # specification part, then the body as a block tree
        stack = [("root", u.body)]
        open_dos: list[Stmt] = []
        pending_dir = None
        in_kernels = False
        while True:
            label, toks, directive = lines[i]
            i += 1
            if toks is None:
                d = directive
                if d.startswith("end kernels"):
                    in_kernels = False
                elif d.startswith("kernels"):
                    in_kernels = True
                elif d.startswith("parallel loop") or d.startswith("parallel"):
                    if not d.startswith("parallel loop"):
                        pending_dir = None  # 'parallel' without loop: region markers only
                    else:
                        pending_dir = d
                elif d.startswith("end parallel"):
                    pending_dir = None
                continue
            words = [t.text for t in toks]
            w0 = words[0]
            if w0 in ("end", "endsubroutine", "endfunction") and (len(words) == 1 or words[1] in (
                    "subroutine", "function")):
                if len(stack) != 1:
                    raise F2CError(f"unclosed block in {name}")
                break
            if w0 in ("use",):
                u.uses.append(words[1])
                continue
            if w0 == "implicit":
                continue
            if w0 in ("real", "integer", "complex", "logical", "character", "double") and not (
                    len(words) > 1 and words[1] == "function"):
                if "=" in words and "::" not in words and w0 != "character":
                    pass  # an assignment to a variable named like a type: not present
                for s in self.parse_decl(toks, scope="local"):
                    if s.name in self.functions or s.name == "rann" and s.name != name:
                        continue  # declares the type of an external function
                    if s.name in u.syms and u.syms[s.name].is_result:
                        continue
                    s.dummy = s.name in args
                    u.syms[s.name] = s
                continue
            if w0 == "parameter":
                for part in split_top(toks[2:-1]):
                    nm = part[0].text
                    u.syms[nm].param = parse_expr(part[2:])
                continue
            st = self.parse_stmt(toks, u)
            st.label = label
            if st.kind == "do":
                st.directive = pending_dir
                pending_dir = None
                stack[-1][1].append(st)
                stack.append(("do", st.body))
                open_dos.append(st)
                continue
            if st.kind == "assign" and in_kernels:
                st.kernels = True
            if st.kind == "if_then" and not st.single:
                stack[-1][1].append(st)
                stack.append(("if", st.branches[-1][1]))
                continue
            if st.kind in ("else_if", "else"):
                kind_, body = stack.pop()
                parent = self._last_if(stack)
                if st.kind == "else":
                    parent.branches.append((None, []))
                else:
                    parent.branches.append((st.cond, []))
                stack.append(("if", parent.branches[-1][1]))
                continue
            if st.kind == "end_if":
                stack.pop()
                continue
            if st.kind == "end_do":
                stack.pop()
                open_dos.pop()
                continue
            stack[-1][1].append(st)
            # a labelled statement ends every open DO with that label (innermost first)
            if label is not None:
                while open_dos and open_dos[-1].end_label == label:
                    open_dos.pop()
                    stack.pop()
        self.units.append(u)
        return i

    @staticmethod
    def _last_if(stack):
        body = stack[-1][1]
        for st in reversed(body):
            if st.kind == "if_then" and not st.single:
                return st
        raise F2CError("else without if")

    def parse_stmt(self, toks, u) -> Stmt:
        words = [t.text for t in toks]
        w0 = words[0]
        if w0 == "do":
            k = 1
            end_label = None
            if toks[1].kind == "num":
                end_label = int(toks[1].text)
                k = 2
            var = toks[k].text
            bounds = split_top(toks[k + 2:])
            return Stmt("do", var=var, lo=parse_expr(bounds[0]), hi=parse_expr(bounds[1]),
                        step=parse_expr(bounds[2]) if len(bounds) > 2 else None,
                        end_label=end_label, body=[])
        if w0 in ("enddo",) or (w0 == "end" and len(words) > 1 and words[1] == "do"):
            return Stmt("end_do")
        if w0 in ("endif",) or (w0 == "end" and len(words) > 1 and words[1] == "if"):
            return Stmt("end_if")
        if w0 == "else" and len(words) > 1 and words[1] == "if":
            return Stmt("else_if", cond=self._if_cond(toks[2:])[0])
        if w0 == "elseif":
            return Stmt("else_if", cond=self._if_cond(toks[1:])[0])
        if w0 == "else":
            return Stmt("else")
        if w0 == "if":
            cond, rest = self._if_cond(toks[1:])
            if [t.text for t in rest] == ["then"]:
                return Stmt("if_then", branches=[(cond, [])], single=False)
            inner = self.parse_stmt(rest, u)
            return Stmt("if_then", branches=[(cond, [inner])], single=True)
        if w0 == "continue":
            return Stmt("continue")
        if w0 in ("goto",) or (w0 == "go" and words[1] == "to"):
            return Stmt("goto", target=int(toks[-1].text))
        if w0 == "return":
            return Stmt("return")
        if w0 == "stop":
            msg = toks[1].text[1:-1] if len(toks) > 1 else ""
            return Stmt("stop", msg=msg)
        if w0 == "call":
            name = words[1]
            args = []
            if len(toks) > 2:
                p = Parser(toks, 3)
                args = p.arglist()
            return Stmt("call", name=name, args=args)
        if w0 in ("open", "close", "read", "write", "print") and len(toks) > 1 and toks[1].text == "(":
            p = Parser(toks, 2)
            ctl = p.arglist()
            items = []
            rest = toks[p.pos:]
            if rest and rest[0].text == ",":
                rest = rest[1:]
            for part in split_top(rest):
                items.append(parse_expr(part))
            return Stmt("io", op=w0, ctl=ctl, items=items)
        if w0 == "format":
            return Stmt("format")
        # assignment
        depth = 0
        for k, t in enumerate(toks):
            depth += t.text == "("
            depth -= t.text == ")"
            if t.text == "=" and depth == 0:
                return Stmt("assign", lhs=parse_expr(toks[:k]), rhs=parse_expr(toks[k + 1:]),
                            kernels=False)
        raise F2CError(f"unknown statement {words}")

    @staticmethod
    def _if_cond(toks):
        depth = 0
        for k, t in enumerate(toks):
            depth += t.text == "("
            depth -= t.text == ")"
            if depth == 0:
                return parse_expr(toks[1:k]), toks[k + 1:]
        raise F2CError("bad if")

    # ---- code generation ----------------------------------------------------------------
    def sym(self, u, name):
        if name in u.syms:
            return u.syms[name]
        if name in self.globals:
            return self.globals[name]
        return None

    def dims_c(self, u, s):
        return [self.gen(u, d)[0] for d in s.dims]

    def var_access(self, u, s):
        """C lvalue of a scalar variable."""
        if s.param is not None and s.scope == "global":
            return s.cname
        if s.dummy and not s.dims:
            return f"(*{s.cname})"
        return s.cname

    @staticmethod
    def flat_index(dims, subs):
        code = f"((long)({subs[-1]})-1)"
        for k in range(len(subs) - 2, -1, -1):
            code = f"((long)({subs[k]})-1) + (long)({dims[k]})*({code})"
        return code

    def gen(self, u, e, ctx=None):
        """(C code, type) of an expression. ctx: elemental loop context {'vars': [...]}."""
        if isinstance(e, Num):
            return e.text, e.t
        if isinstance(e, Str):
            body = e.text[1:-1].replace("''", "'").replace('"', '\\"')
            return f'"{body}"', "ch"
        if isinstance(e, Cplx):
            a, _ = self.gen(u, e.re, ctx)
            b, _ = self.gen(u, e.im, ctx)
            return f"__builtin_complex((double)({a}), (double)({b}))", "c8"
        if isinstance(e, Un):
            a, t = self.gen(u, e.a, ctx)
            if e.op == "!":
                return f"(!{a})", "l"
            return (f"(-{a})" if e.op == "-" else f"(+{a})"), t
        if isinstance(e, Bin):
            return self.gen_bin(u, e, ctx)
        if isinstance(e, Name):
            s = self.sym(u, e.name)
            if s is None:
                raise F2CError(f"unknown name {e.name} in {u.name}")
            if s.dims:
                if ctx is None:
                    raise F2CError(f"whole array {e.name} outside an array context in {u.name}")
                subs = list(ctx["vars"])
                if len(subs) != len(s.dims):
                    raise F2CError(f"rank mismatch for {e.name} in {u.name}")
                self._shape_check(ctx, self.dims_c(u, s), e.name)
                return f"{s.cname}[{self.flat_index(self.dims_c(u, s), subs)}]", s.t
            if s.param is not None and s.scope == "local":
                return s.cname, s.t
            return self.var_access(u, s), s.t
        if isinstance(e, Ref):
            return self.gen_ref(u, e, ctx)
        raise F2CError(f"cannot generate {e}")

    def _shape_check(self, ctx, extents, what):
        if ctx.get("extents") is not None and len(ctx["extents"]) == len(extents):
            if [x.replace(" ", "") for x in ctx["extents"]] != [x.replace(" ", "") for x in extents]:
                raise F2CError(f"non-conformable array {what}: {extents} vs {ctx['extents']}")

    def gen_bin(self, u, e, ctx):
        a, ta = self.gen(u, e.a, ctx)
        op = e.op
        if op == "**":
            if isinstance(e.b, Num) and e.b.t == "i4" and 1 <= int(e.b.text) <= 4:
                n = int(e.b.text)
                tmp = f"({a})"
                return "(" + "*".join([tmp] * n) + ")", ta
            b, tb = self.gen(u, e.b, ctx)
            if tb in ("i4", "i8"):
                fn = {"r8": "f2c_powi_r8", "r4": "f2c_powi_r4", "i4": "f2c_powi_i4"}[ta]
                return f"{fn}({a}, {b})", ta
            t = ORDER[max(ORDER.index(ta), ORDER.index(tb))]
            if t == "c8":
                raise F2CError("complex power not supported")
            if t == "r4":
                return f"powf({a}, {b})", "r4"
            return f"pow((double)({a}), (double)({b}))", "r8"
        b, tb = self.gen(u, e.b, ctx)
        cmp = {".eq.": "==", ".ne.": "!=", ".lt.": "<", ".le.": "<=", ".gt.": ">", ".ge.": ">=",
               "==": "==", "/=": "!=", "<": "<", "<=": "<=", ">": ">", ">=": ">="}
        if op in cmp:
            return f"({a} {cmp[op]} {b})", "l"
        if op == ".and.":
            return f"({a} && {b})", "l"
        if op == ".or.":
            return f"({a} || {b})", "l"
        t = ORDER[max(ORDER.index(ta), ORDER.index(tb))]
        return f"({a} {op} {b})", t

    def gen_ref(self, u, e, ctx):
        name = e.name
        s = self.sym(u, name)
        if s is not None and s.dims:
            dims = self.dims_c(u, s)
            subs, extents, k = [], [], 0
            for d, a in zip(dims, e.args):
                if isinstance(a, Slice):
                    if a.lo is not None or a.hi is not None:
                        raise F2CError(f"partial section of {name} outside sum() in {u.name}")
                    if ctx is None:
                        raise F2CError(f"section {name} outside an array context")
                    subs.append(ctx["vars"][k])
                    extents.append(d)
                    k += 1
                else:
                    subs.append(self.gen(u, a, None)[0])
            if extents:
                if k != len(ctx["vars"]):
                    raise F2CError(f"section rank mismatch for {name}")
                self._shape_check(ctx, extents, name)
            return f"{s.cname}[{self.flat_index(dims, subs)}]", s.t
        # intrinsics
        args = e.args
        if name in ("dble", "dfloat"):
            a, t = self.gen(u, args[0], ctx)
            return (f"creal({a})" if t == "c8" else f"((double)({a}))"), "r8"
        if name == "real":
            a, t = self.gen(u, args[0], ctx)
            if t == "c8":
                return f"creal({a})", "r8"
            return f"((float)({a}))", "r4"
        if name == "int":
            a, _ = self.gen(u, args[0], ctx)
            return f"((int)({a}))", "i4"
        if name in ("sqrt", "dsqrt"):
            a, t = self.gen(u, args[0], ctx)
            return ({"r4": f"sqrtf({a})", "c8": f"csqrt({a})"}.get(t, f"sqrt({a})")), ("r4" if t == "r4" else "r8" if t != "c8" else "c8")
        if name in ("exp", "dexp"):
            a, t = self.gen(u, args[0], ctx)
            return (f"expf({a})" if t == "r4" else f"exp({a})"), ("r4" if t == "r4" else "r8")
        if name in ("cos", "dcos", "sin", "dsin"):
            a, t = self.gen(u, args[0], ctx)
            fn = name.lstrip("d")
            return (f"{fn}f({a})" if t == "r4" else f"{fn}({a})"), ("r4" if t == "r4" else "r8")
        if name in ("abs", "dabs", "cdabs"):
            a, t = self.gen(u, args[0], ctx)
            if t == "c8":
                return f"cabs({a})", "r8"
            if t in ("i4", "i8"):
                return f"llabs({a})", t
            return (f"fabsf({a})" if t == "r4" else f"fabs({a})"), t
        if name == "iand":
            a, ta = self.gen(u, args[0], ctx)
            b, tb = self.gen(u, args[1], ctx)
            return f"({a} & {b})", "i4"
        if name == "mod":
            a, ta = self.gen(u, args[0], ctx)
            b, tb = self.gen(u, args[1], ctx)
            return f"({a} % {b})", ta
        if name == "sum":
            return self.gen_sum(u, args[0])
        if name in self.functions:
            return self.call_expr(u, name, args, ctx), self.functions[name]
        if name in EXTERNALS:
            rtype, kinds = EXTERNALS[name]
            cargs = []
            for a, kd in zip(args, kinds):
                if kd == "v":
                    cargs.append(self.gen(u, a, None)[0])
                else:
                    cargs.append(self.actual_arg(u, a))
            return f"{name}({', '.join(cargs)})", "i4"
        raise F2CError(f"unknown function or array {name} in {u.name}")

    def gen_sum(self, u, a):
        if not (isinstance(a, Ref) and len(a.args) == 1 and isinstance(a.args[0], Slice)):
            raise F2CError("sum() supports one 1-D section")
        s = self.sym(u, a.name)
        lo = self.gen(u, a.args[0].lo, None)[0] if a.args[0].lo is not None else "1"
        hi = self.gen(u, a.args[0].hi, None)[0] if a.args[0].hi is not None else self.dims_c(u, s)[0]
        fn = {"r8": "f2c_sum_r8", "r4": "f2c_sum_r4"}[s.t]
        return f"{fn}({s.cname}, {lo}, {hi})", s.t

    def actual_arg(self, u, a):
        """C pointer expression passing actual argument `a` by reference."""
        if isinstance(a, Name):
            s = self.sym(u, a.name)
            if s is None:
                raise F2CError(f"unknown actual argument {a.name}")
            if s.dims or s.t == "ch":
                return s.cname
            if s.dummy:
                return s.cname
            if s.param is not None:
                return f"&({CTYPE[s.t]}){{{self.gen(u, a)[0]}}}"
            return f"&{s.cname}"
        if isinstance(a, Ref):
            s = self.sym(u, a.name)
            if s is not None and s.dims:
                code, _ = self.gen(u, a)
                return f"&{code}"
        code, t = self.gen(u, a)
        return f"&({CTYPE[t]}){{{code}}}"

    def call_expr(self, u, name, args, ctx=None):
        return f"f_{name}({', '.join(self.actual_arg(u, a) for a in args)})"

    # ---- statements ---------------------------------------------------------------------
    def emit_unit(self, u):
        out = []
        params = ", ".join(f"void* {a}_" for a in u.args) or "void"
        ret = CTYPE[u.rtype] if u.kind == "fun" else "void"
        out.append(f"{ret} f_{u.name}({params}) {{")
        for a in u.args:
            s = u.syms.get(a)
            if s is None:
                raise F2CError(f"undeclared dummy {a} in {u.name}")
            out.append(f"  {CTYPE[s.t]}* f_{a} = ({CTYPE[s.t]}*){a}_;")
        for s in u.syms.values():
            if s.dummy:
                continue
            if s.param is not None:
                out.append(f"  const {CTYPE[s.t]} {s.cname} = {self.gen(u, s.param)[0]};")
            elif s.t == "ch":
                out.append(f"  char {s.cname}[{s.charlen + 1}] = {{0}};")
            elif s.dims:
                size = "*".join(f"({d})" for d in self.dims_c(u, s))
                out.append(f"  static {CTYPE[s.t]} {s.cname}[{size}];")
            else:
                out.append(f"  {CTYPE[s.t]} {s.cname} = 0;")
        for st in u.body:
            out.extend(self.emit_stmt(u, st, 1))
        if u.kind == "fun":
            out.append(f"  return {u.syms[u.name].cname};")
        out.append("}")
        return out

    def emit_block(self, u, body, ind):
        out = []
        for st in body:
            out.extend(self.emit_stmt(u, st, ind))
        return out

    def emit_stmt(self, u, st, ind):
        p = "  " * ind
        out = []
        k = st.kind
        if k == "do":
            var = self.var_access(u, u.syms[st.var])
            lo = self.gen(u, st.lo)[0]
            hi = self.gen(u, st.hi)[0]
            step = self.gen(u, st.step)[0] if st.step is not None else "1"
            pragma = self.omp_pragma(u, st)
            if pragma:
                out.append(p + pragma)
            out.append(f"{p}for ({var} = {lo}; {var} <= {hi}; {var} += {step}) {{")
            out.extend(self.emit_block(u, st.body, ind + 1))
            out.append(p + "}")
            return out
        if k == "if_then":
            for n, (cond, body) in enumerate(st.branches):
                if cond is None:
                    out.append(p + "} else {")
                else:
                    c = self.gen(u, cond)[0]
                    out.append(p + ("if" if n == 0 else "} else if") + f" ({c}) {{")
                out.extend(self.emit_block(u, body, ind + 1))
            out.append(p + "}")
            return out
        lab = f"L{st.label}: " if st.label is not None else ""
        if k == "continue":
            return [f"{p}{lab};"]
        if k == "format":
            return [f"{p}{lab}; /* format */"] if lab else []
        if k == "goto":
            return [f"{p}{lab}goto L{st.target};"]
        if k == "return":
            if u.kind == "fun":
                return [f"{p}{lab}return {u.syms[u.name].cname};"]
            return [f"{p}{lab}return;"]
        if k == "stop":
            return [f'{p}{lab}f2c_stop("{st.msg}");']
        if k == "call":
            if st.name == "flush":
                return [f"{p}{lab}f2c_flush({self.gen(u, st.args[0])[0]});"]
            return [f"{p}{lab}{self.call_expr(u, st.name, st.args)};"]
        if k == "io":
            return [p + lab + line for line in self.emit_io(u, st)]
        if k == "assign":
            return [p + lab + line if i == 0 else p + line
                    for i, line in enumerate(self.emit_assign(u, st))]
        raise F2CError(f"cannot emit {k}")

    def lhs_shape(self, u, lhs):
        """None for a scalar target, else the list of section extents."""
        if isinstance(lhs, Name):
            s = self.sym(u, lhs.name)
            return self.dims_c(u, s) if s.dims else None
        if isinstance(lhs, Ref):
            s = self.sym(u, lhs.name)
            if s is None or not s.dims:
                raise F2CError(f"bad assignment target {lhs.name}")
            dims = self.dims_c(u, s)
            ext = [d for d, a in zip(dims, lhs.args) if isinstance(a, Slice)]
            return ext or None
        raise F2CError("bad assignment target")

    def emit_assign(self, u, st):
        shape = self.lhs_shape(u, st.lhs)
        if shape is None:
            lhs, tl = self.gen(u, st.lhs)
            rhs, tr = self.gen(u, st.rhs)
            return [f"{lhs} = ({CTYPE[tl]})({rhs});" if tl != "c8" else f"{lhs} = {rhs};"]
        self.tmp += 1
        vars_ = [f"f2c_s{self.tmp}_{d}" for d in range(len(shape))]
        ctx = {"vars": vars_, "extents": shape}
        lhs, tl = self.gen(u, st.lhs, ctx)
        rhs, tr = self.gen(u, st.rhs, ctx)
        lines = []
        if st.kernels:
            lines.append(f"#pragma omp parallel for collapse({len(shape)})" if len(shape) > 1
                         else "#pragma omp parallel for")
        # loops: last dimension outermost (array-element order)
        depth = 0
        for d in reversed(range(len(shape))):
            lines.append("  " * depth + f"for (long {vars_[d]} = 1; {vars_[d]} <= {shape[d]}; ++{vars_[d]})")
            depth += 1
        conv = f"({CTYPE[tl]})({rhs})" if tl != "c8" else rhs
        lines.append("  " * depth + f"{lhs} = {conv};")
        return lines

    def emit_io(self, u, st):
        ctl = st.ctl
        op = st.op
        pos = [a for a in ctl if not (isinstance(a, tuple) and a[0] == "kw")]
        kw = {a[1]: a[2] for a in ctl if isinstance(a, tuple) and a[0] == "kw"}
        unit = kw.get("unit", pos[0] if pos else None)
        if op == "open":
            u_c = self.gen(u, unit)[0]
            f = kw["file"]
            f_c = self.gen(u, f)[0] if not isinstance(f, Name) else self.sym(u, f.name).cname
            form = kw.get("form")
            formatted = 0 if (isinstance(form, Str) and "unformatted" in form.text.lower()) else 1
            return [f"f2c_open({u_c}, {f_c}, {formatted});"]
        if op == "close":
            return [f"f2c_close({self.gen(u, unit)[0]});"]
        fmt = kw.get("fmt", pos[1] if len(pos) > 1 else None)
        # internal write: the unit is a character variable
        if isinstance(unit, Name) and self.sym(u, unit.name) is not None and self.sym(u, unit.name).t == "ch":
            s = self.sym(u, unit.name)
            vals = [self.gen(u, it)[0] for it in st.items]
            fmt_c = self.gen(u, fmt)[0]
            arr = ", ".join(f"(long long)({v})" for v in vals) or "0"
            return [f"f2c_write_internal({s.cname}, {s.charlen}, {fmt_c}, {len(vals)}, "
                    f"(const long long[]){{{arr}}});"]
        u_c = self.gen(u, unit)[0]
        if isinstance(unit, Num) and unit.text == "6":
            return ["; /* console output (unit 6) */"]
        if op == "read":
            if fmt is None:  # unformatted: whole arrays
                return [f"f2c_read_unf({u_c}, {self.sym(u, it.name).cname}, (long)sizeof(*{self.sym(u, it.name).cname})*"
                        + "*".join(f"({d})" for d in self.dims_c(u, self.sym(u, it.name))) + ");"
                        for it in st.items]
            types, ptrs = "", []
            for it in st.items:
                s = self.sym(u, it.name)
                types += {"i4": "i", "i8": "I", "r4": "f", "r8": "d"}[s.t]
                ptrs.append(s.cname if s.dummy else f"&{s.cname}")
            return [f'f2c_read_list({u_c}, "{types}", {", ".join(ptrs)});']
        if op == "write":
            if fmt is None:
                return [f"f2c_write_unf({u_c}, {self.sym(u, it.name).cname}, (long)sizeof(*{self.sym(u, it.name).cname})*"
                        + "*".join(f"({d})" for d in self.dims_c(u, self.sym(u, it.name))) + ");"
                        for it in st.items]
            written, fp64 = [], []
            for it in st.items:
                c, _ = self.gen(u, it)
                written.append(f"(double)({c})")
                if isinstance(it, Ref) and it.name == "real" and self.sym(u, "real") is None:
                    fp64.append(f"(double)({self.gen(u, it.args[0])[0]})")
                else:
                    fp64.append(f"(double)({c})")
            n = len(written)
            return [f"f2c_write_vals({u_c}, {n}, (const double[]){{{', '.join(written)}}}, "
                    f"(const double[]){{{', '.join(fp64)}}});"]
        raise F2CError(f"unsupported I/O {op}")

    # ---- OpenACC parallel loops -> OpenMP -------------------------------------------------
    def omp_pragma(self, u, st):
        d = st.directive
        if not d or " seq" in f" {d}" or not d.startswith("parallel loop"):
            return None
        m = re.search(r"collapse\((\d+)\)", d)
        ncol = int(m.group(1)) if m else 1
        loops = [st]
        cur = st
        for _ in range(ncol - 1):
            if len(cur.body) < 1 or cur.body[0].kind != "do":
                return None
            inner = [x for x in cur.body if x.kind not in ("continue",)]
            if len(inner) != 1:
                return None
            cur = cur.body[0]
            loops.append(cur)
        loop_vars = {lp.var for lp in loops}
        assigned, unsafe = set(), [False]

        def scan(body):
            for s in body:
                if s.kind == "call" and s.name != "flush":
                    unsafe[0] = True
                if s.kind in ("io", "stop"):
                    unsafe[0] = True
                if s.kind == "do":
                    assigned.add(s.var)
                    scan(s.body)
                if s.kind == "if_then":
                    for cond, b in s.branches:
                        if cond is not None and self._calls_function(cond):
                            unsafe[0] = True
                        scan(b)
                if s.kind == "assign":
                    if self._calls_function(s.rhs):
                        unsafe[0] = True
                    lhs = s.lhs
                    if isinstance(lhs, Name):
                        sym = self.sym(u, lhs.name)
                        if sym.dims:
                            unsafe[0] = True  # whole-array write inside a parallel loop
                        else:
                            if self._mentions(s.rhs, lhs.name):
                                unsafe[0] = True  # accumulation into a shared scalar
                            assigned.add(lhs.name)
                    else:
                        subs = {a.name for a in lhs.args if isinstance(a, Name)}
                        if not loop_vars <= subs and not any(isinstance(a, Slice) for a in lhs.args):
                            unsafe[0] = True  # indirect index: iterations may collide
                        if any(isinstance(a, Slice) for a in lhs.args) and not loop_vars <= subs:
                            unsafe[0] = True

        scan(loops[-1].body)
        if unsafe[0]:
            return None
        priv = sorted(n for n in assigned - loop_vars)
        for n in priv:
            s = self.sym(u, n)
            if s is None or s.dims or s.dummy or s.scope == "global":
                return None
        clause = f" private({', '.join('f_' + n for n in priv)})" if priv else ""
        col = f" collapse({ncol})" if ncol > 1 else ""
        return f"#pragma omp parallel for{col}{clause}"

    def _calls_function(self, e):
        if isinstance(e, Ref):
            if e.name in self.functions:
                return True
            return any(self._calls_function(a) for a in e.args if not isinstance(a, (Slice, tuple)))
        if isinstance(e, Bin):
            return self._calls_function(e.a) or self._calls_function(e.b)
        if isinstance(e, Un):
            return self._calls_function(e.a)
        return False

    def _mentions(self, e, name):
        if isinstance(e, Name):
            return e.name == name
        if isinstance(e, Ref):
            return e.name == name or any(self._mentions(a, name) for a in e.args
                                         if not isinstance(a, (Slice, tuple)))
        if isinstance(e, Bin):
            return self._mentions(e.a, name) or self._mentions(e.b, name)
        if isinstance(e, Un):
            return self._mentions(e.a, name)
        if isinstance(e, Cplx):
            return self._mentions(e.re, name) or self._mentions(e.im, name)
        return False

    # ---- whole file ---------------------------------------------------------------------
    def emit(self, sources):
        out = ["/* Generated by oracle/f2c_ref.py from the reference's Fortran sources:",
               *[f" *   {s}" for s in sources],
               " * Test infrastructure only (oracle/_ref, never committed, never linked into the",
               " * product). Regenerate instead of editing. */",
               "#include <complex.h>", "#include <math.h>", "#include <setjmp.h>",
               '#include "f2c_rt.h"', ""]
        # parameters (integer parameters overridable by -DF2C_<NAME>)
        unit0 = Unit("sub", "__globals__", [])
        for s in self.globals.values():
            if s.param is None:
                continue
            val = self.gen(unit0, s.param)[0]
            if s.t in ("i4", "i8"):
                out.append(f"#ifdef F2C_{s.name.upper()}")
                out.append(f"#define {s.cname} (F2C_{s.name.upper()})")
                out.append("#else")
                out.append(f"#define {s.cname} ({val})")
                out.append("#endif")
            else:
                out.append(f"#define {s.cname} ({val})")
        out.append("")
        for s in self.globals.values():
            if s.param is not None:
                continue
            if s.dims:
                size = "*".join(f"({self.gen(unit0, d)[0]})" for d in s.dims)
                out.append(f"{CTYPE[s.t]} {s.cname}[{size}];")
            else:
                out.append(f"{CTYPE[s.t]} {s.cname};")
        out.append("")
        for uu in self.units:
            ret = CTYPE[uu.rtype] if uu.kind == "fun" else "void"
            params = ", ".join(f"void* {a}_" for a in uu.args) or "void"
            out.append(f"{ret} f_{uu.name}({params});")
        out.append("")
        for uu in self.units:
            out.extend(self.emit_unit(uu))
            out.append("")
        # exported wrappers: a Fortran STOP returns 1 instead of ending the process
        for uu in self.units:
            if uu.kind != "sub":
                continue
            params = ", ".join(f"void* a{k}" for k in range(len(uu.args))) or "void"
            call = ", ".join(f"a{k}" for k in range(len(uu.args)))
            out.append(f"int ref_{uu.name}({params}) {{")
            out.append("  if (setjmp(f2c_stop_env)) return 1;")
            out.append(f"  f_{uu.name}({call});")
            out.append("  return 0;")
            out.append("}")
        # sizes of the compiled grid
        out.append("int ref_grid(int* nx, int* ny) { *nx = f_nx; *ny = f_ny; return 0; }")
        return "\n".join(out) + "\n"


def translate(src_dir: str, files=REF_FILES) -> str:
    tr = Translator()
    paths = [os.path.join(src_dir, f) for f in files]
    for path in paths:
        with open(path, encoding="latin-1") as f:
            text = f.read()
        try:
            tr.parse_file(text)
        except F2CError as e:
            raise F2CError(f"{os.path.basename(path)}: {e}") from None
    try:
        return tr.emit([os.path.relpath(p, os.path.dirname(src_dir)) for p in paths])
    except F2CError as e:
        raise F2CError(f"emit: {e}") from None


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--src", default=os.environ.get("GTURBO_REF_SRC", DEFAULT_SRC))
    ap.add_argument("--out", default=os.path.join(os.path.dirname(os.path.abspath(__file__)), "_ref",
                                                  "gturbo_ref.c"))
    a = ap.parse_args(argv)
    code = translate(a.src)
    os.makedirs(os.path.dirname(a.out), exist_ok=True)
    with open(a.out, "w") as f:
        f.write(code)
    print(a.out)
    return 0


if __name__ == "__main__":
    sys.exit(main())
