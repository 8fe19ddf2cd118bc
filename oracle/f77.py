"""A Fortran 77 subset executor -- test infrastructure for the oracle.

It runs Fortran 77 source files (fixed form, the subset that Nekbone's
solver sources use) by translating each program unit into a Python function
and executing it.  It exists to produce golden vectors from the reference's
own Fortran sources where no Fortran compiler is available; nothing in the
product imports it.

Semantics follow gfortran with ``-fdefault-real-8`` on x86-64 without FMA
contraction: every REAL (and real constant) is an IEEE double, and each
arithmetic operation rounds once, in source order (Python floats have the
same semantics).  Default INTEGERs are 32-bit: products of two of them wrap.
Integer division truncates toward zero.  ``x**n`` with an integer exponent
multiplies as libgcc's ``__powidf2`` does.

Supported: SUBROUTINE / FUNCTION units; IMPLICIT, type declarations with
array bounds (lower bounds, assumed size), DIMENSION, COMMON (storage
association by position), PARAMETER, DATA, SAVE, EXTERNAL; assignment, CALL,
block IF / ELSE IF / ELSE, logical IF, DO with or without a terminal label
(shared terminals too), DO WHILE, CONTINUE, GOTO (forward and backward, by
exception), RETURN, STOP; I/O statements are ignored.  C preprocessor
#ifdef / #ifndef / #else / #endif and INCLUDE are resolved when the source
is read.  Arguments are passed by reference (``Ref``: a list and an offset);
scalar dummies are copied in at entry and out at exit.

Routines the sources call but do not define are looked up in ``externals``
(Python callables receiving ``Ref`` arguments).
"""
from __future__ import annotations

import math
import re
from pathlib import Path


class F77Error(RuntimeError):
    pass


class Ref:
    """A reference to storage: element ``o`` of list ``b``."""

    __slots__ = ("b", "o")

    def __init__(self, b, o=0):
        self.b = b
        self.o = o


class _Goto(Exception):
    def __init__(self, label):
        self.label = label


class _Return(Exception):
    pass


class _Stop(Exception):
    pass


# ----------------------------------------------------------------- source --
def _cpp(lines, defines):
    out, stack = [], []
    for ln in lines:
        s = ln.strip()
        if s.startswith("#"):
            parts = s[1:].split()
            d = parts[0] if parts else ""
            if d == "ifdef":
                stack.append(parts[1] in defines)
            elif d == "ifndef":
                stack.append(parts[1] not in defines)
            elif d == "else":
                stack[-1] = not stack[-1]
            elif d == "endif":
                stack.pop()
            out.append("")
            continue
        out.append(ln if all(stack) else "")
    return out


def _strip_comment(text):
    """Removes a trailing ! comment outside string literals."""
    q = False
    for i, ch in enumerate(text):
        if ch == "'":
            q = not q
        elif ch == "!" and not q:
            return text[:i]
    return text


def _lower_outside_strings(text):
    out, q = [], False
    for ch in text:
        if ch == "'":
            q = not q
        out.append(ch if q else ch.lower())
    return "".join(out)


def read_statements(path, include_dirs, defines=(), overrides=None):
    """Fixed-form statements of a file: list of (label, text, origin)."""
    overrides = overrides or {}

    def load(p):
        name = Path(p).name
        if name in overrides:
            return overrides[name].splitlines()
        return Path(p).read_text(errors="replace").splitlines()

    def expand(lines, origin):
        res = []
        for i, ln in enumerate(_cpp(lines, set(defines))):
            m = re.match(r"^\s+include\s+'([^']+)'", ln, re.I)
            if m and not ln[:1].lower() in ("c", "*", "!"):
                inc = m.group(1)
                src = None
                if inc in overrides:
                    src = overrides[inc].splitlines()
                else:
                    for d in include_dirs:
                        if (Path(d) / inc).exists():
                            src = load(Path(d) / inc)
                            break
                if src is None:
                    raise F77Error(f"include '{inc}' not found")
                res.extend(expand(src, f"{inc}"))
            else:
                res.append((ln, f"{origin}:{i + 1}"))
        return res

    raw = expand(load(path), Path(path).name)
    stmts = []
    for ln, origin in raw:
        ln = ln.expandtabs(6) if ln.startswith("\t") else ln
        if not ln.strip():
            continue
        if ln[0] in "cC*!":
            continue
        if ln.lstrip().startswith("!"):
            continue
        body = ln[:72]
        lab = body[:5].strip()
        cont = len(body) > 5 and body[5] not in (" ", "0")
        text = _strip_comment(body[6:])
        if cont:
            if not stmts:
                raise F77Error(f"continuation without a statement at {origin}")
            stmts[-1][1] += text
        else:
            stmts.append([lab, text, origin])
    out = []
    for lab, text, origin in stmts:
        t = _lower_outside_strings(text).strip()
        if t:
            out.append((int(lab) if lab else None, t, origin))
    return out


# ------------------------------------------------------------------ lexer --
_DOTOPS = {".eq.": "==", ".ne.": "!=", ".lt.": "<", ".le.": "<=", ".gt.": ">",
           ".ge.": ">=", ".and.": "and", ".or.": "or", ".not.": "not",
           ".true.": "TRUE", ".false.": "FALSE", ".eqv.": "eqv", ".neqv.": "neqv"}


def tokenize(s):
    toks, i, n = [], 0, len(s)
    while i < n:
        ch = s[i]
        if ch == " ":
            i += 1
            continue
        if ch == "'":
            j, buf = i + 1, []
            while True:
                if j >= n:
                    raise F77Error(f"unterminated string in {s!r}")
                if s[j] == "'":
                    if j + 1 < n and s[j + 1] == "'":
                        buf.append("'")
                        j += 2
                        continue
                    break
                buf.append(s[j])
                j += 1
            toks.append(("str", "".join(buf)))
            i = j + 1
            continue
        if ch == ".":
            m = re.match(r"\.(eq|ne|lt|le|gt|ge|and|or|not|true|false|eqv|neqv)\.", s[i:])
            if m:
                toks.append(("op", _DOTOPS[m.group(0)]))
                i += len(m.group(0))
                continue
        if ch.isdigit() or (ch == "." and i + 1 < n and s[i + 1].isdigit()):
            j = i
            while j < n and s[j].isdigit():
                j += 1
            is_real = False
            if j < n and s[j] == "." and not re.match(
                    r"\.(eq|ne|lt|le|gt|ge|and|or|not|true|false|eqv|neqv)\.", s[j:]):
                is_real = True
                j += 1
                while j < n and s[j].isdigit():
                    j += 1
            m = re.match(r"[eEdD][+-]?\d+", s[j:])
            if m:
                is_real = True
                j += len(m.group(0))
            txt = s[i:j]
            if is_real:
                toks.append(("real", float(txt.replace("d", "e").replace("D", "e"))))
            else:
                toks.append(("int", int(txt)))
            i = j
            continue
        if ch.isalpha() or ch == "_":
            j = i
            while j < n and (s[j].isalnum() or s[j] in "_$"):
                j += 1
            toks.append(("id", s[i:j]))
            i = j
            continue
        if s.startswith("**", i):
            toks.append(("op", "**"))
            i += 2
            continue
        if s.startswith("//", i):
            toks.append(("op", "//"))
            i += 2
            continue
        if s.startswith("==", i) or s.startswith("/=", i) or s.startswith("<=", i) or \
                s.startswith(">=", i):
            toks.append(("op", {"==": "==", "/=": "!=", "<=": "<=", ">=": ">="}[s[i:i + 2]]))
            i += 2
            continue
        if ch in "+-*/(),=:<>":
            toks.append(("op", ch))
            i += 1
            continue
        raise F77Error(f"unexpected character {ch!r} in {s!r}")
    return toks


# ----------------------------------------------------------------- parser --
class Expr:
    pass


class Num(Expr):
    def __init__(self, v):
        self.v = v


class Str(Expr):
    def __init__(self, v):
        self.v = v


class Bool(Expr):
    def __init__(self, v):
        self.v = v


class Name(Expr):
    def __init__(self, name):
        self.name = name


class Apply(Expr):        # name(args): array element or function call
    def __init__(self, name, args):
        self.name = name
        self.args = args


class BinOp(Expr):
    def __init__(self, op, a, b):
        self.op, self.a, self.b = op, a, b


class UnOp(Expr):
    def __init__(self, op, a):
        self.op, self.a = op, a


class Parser:
    def __init__(self, toks):
        self.t = toks
        self.i = 0

    def peek(self, k=0):
        j = self.i + k
        return self.t[j] if j < len(self.t) else (None, None)

    def take(self, val=None):
        tok = self.peek()
        if val is not None and tok[1] != val:
            raise F77Error(f"expected {val!r}, got {tok!r}")
        self.i += 1
        return tok

    def at_end(self):
        return self.i >= len(self.t)

    def expr(self):
        return self.eqv()

    def eqv(self):
        a = self.or_()
        while self.peek()[1] in ("eqv", "neqv"):
            op = self.take()[1]
            a = BinOp(op, a, self.or_())
        return a

    def or_(self):
        a = self.and_()
        while self.peek()[1] == "or":
            self.take()
            a = BinOp("or", a, self.and_())
        return a

    def and_(self):
        a = self.not_()
        while self.peek()[1] == "and":
            self.take()
            a = BinOp("and", a, self.not_())
        return a

    def not_(self):
        if self.peek()[1] == "not":
            self.take()
            return UnOp("not", self.not_())
        return self.rel()

    def rel(self):
        a = self.concat()
        if self.peek()[1] in ("==", "!=", "<", "<=", ">", ">="):
            op = self.take()[1]
            a = BinOp(op, a, self.concat())
        return a

    def concat(self):
        a = self.add()
        while self.peek()[1] == "//":
            self.take()
            a = BinOp("//", a, self.add())
        return a

    def add(self):
        if self.peek()[1] in ("+", "-"):
            op = self.take()[1]
            a = self.mul()
            a = UnOp(op, a)
        else:
            a = self.mul()
        while self.peek()[1] in ("+", "-"):
            op = self.take()[1]
            a = BinOp(op, a, self.mul())
        return a

    def mul(self):
        a = self.power()
        while self.peek()[1] in ("*", "/"):
            op = self.take()[1]
            a = BinOp(op, a, self.power())
        return a

    def power(self):
        a = self.primary()
        if self.peek()[1] == "**":
            self.take()
            if self.peek()[1] in ("+", "-"):
                op = self.take()[1]
                b = UnOp(op, self.power())
            else:
                b = self.power()
            return BinOp("**", a, b)
        return a

    def primary(self):
        kind, v = self.peek()
        if kind == "int" or kind == "real":
            self.take()
            return Num(v)
        if kind == "str":
            self.take()
            return Str(v)
        if kind == "op" and v in ("TRUE", "FALSE"):
            self.take()
            return Bool(v == "TRUE")
        if kind == "op" and v == "(":
            self.take()
            e = self.expr()
            self.take(")")
            return e
        if kind == "id":
            self.take()
            if self.peek()[1] == "(":
                self.take()
                args = []
                if self.peek()[1] != ")":
                    while True:
                        args.append(self.expr())
                        if self.peek()[1] == ",":
                            self.take()
                            continue
                        break
                self.take(")")
                return Apply(v, args)
            return Name(v)
        raise F77Error(f"unexpected token {self.peek()!r}")


def parse_expr(text):
    p = Parser(tokenize(text))
    e = p.expr()
    if not p.at_end():
        raise F77Error(f"trailing tokens in expression {text!r}")
    return e


def _split_top(text, sep=","):
    parts, depth, q, cur = [], 0, False, []
    for ch in text:
        if ch == "'":
            q = not q
        if not q:
            if ch == "(":
                depth += 1
            elif ch == ")":
                depth -= 1
            elif ch == sep and depth == 0:
                parts.append("".join(cur))
                cur = []
                continue
        cur.append(ch)
    parts.append("".join(cur))
    return [p.strip() for p in parts]


def _find_top(text, ch):
    depth, q = 0, False
    for i, c in enumerate(text):
        if c == "'":
            q = not q
        if q:
            continue
        if c == "(":
            depth += 1
        elif c == ")":
            depth -= 1
        elif c == ch and depth == 0:
            return i
    return -1


def _match_paren(text, start):
    depth, q = 0, False
    for i in range(start, len(text)):
        c = text[i]
        if c == "'":
            q = not q
        if q:
            continue
        if c == "(":
            depth += 1
        elif c == ")":
            depth -= 1
            if depth == 0:
                return i
    raise F77Error(f"unbalanced parentheses in {text!r}")


# statements
class Stmt:
    label = None
    origin = ""


class SAssign(Stmt):
    def __init__(self, target, expr):
        self.target, self.expr = target, expr


class SCall(Stmt):
    def __init__(self, name, args):
        self.name, self.args = name, args


class SIf(Stmt):
    def __init__(self, branches, else_body):
        self.branches, self.else_body = branches, else_body  # [(cond, body)]


class SDo(Stmt):
    def __init__(self, var, start, end, step, body, while_cond=None):
        self.var, self.start, self.end, self.step, self.body = var, start, end, step, body
        self.while_cond = while_cond


class SGoto(Stmt):
    def __init__(self, target):
        self.target = target


class SSimple(Stmt):
    def __init__(self, kind):
        self.kind = kind  # continue, return, stop, nop


TYPE_WORDS = [("double precision", "r8"), ("real*8", "r8"), ("real*4", "r4"), ("real", "r8"),
              ("integer*8", "i8"), ("integer*4", "i4"), ("integer", "i4"),
              ("logical", "l"), ("character", "c"), ("complex", "cx")]


class Unit:
    def __init__(self, kind, name, args, rtype):
        self.kind, self.name, self.args, self.rtype = kind, name, args, rtype
        self.decls = []   # (kind, text, origin)
        self.body = []    # flat executable statements (label, text, origin)
        self.tree = None


def split_units(stmts):
    units, cur = [], None
    for lab, text, origin in stmts:
        if cur is None:
            m = re.match(r"^(?:(double precision|real\*8|real|integer\*8|integer|logical)\s+)?"
                         r"(subroutine|function)\s+([a-z_]\w*)\s*(\((.*)\))?\s*$", text)
            if m:
                rtype = dict(TYPE_WORDS).get(m.group(1)) if m.group(1) else None
                args = [a for a in _split_top(m.group(5))] if m.group(5) else []
                args = [a for a in args if a]
                cur = Unit(m.group(2), m.group(3), args, rtype)
                continue
            if re.match(r"^program\s", text) or re.match(r"^block\s*data", text):
                cur = Unit("program", text.split()[1] if len(text.split()) > 1 else "main",
                           [], None)
                continue
            raise F77Error(f"statement outside a program unit at {origin}: {text!r}")
        if re.match(r"^end\s*(subroutine|function|program)?(\s+\w+)?$", text) and \
                not re.match(r"^end\s*(if|do)\b", text):
            units.append(cur)
            cur = None
            continue
        cur.body.append((lab, text, origin))
    if cur is not None:
        raise F77Error(f"unit {cur.name} has no END")
    return units


_DECL_RE = re.compile(
    r"^(implicit|double precision|real\*8|real\*4|real|integer\*8|integer\*4|integer|logical|"
    r"character(\*\d+|\*\(\*\))?|complex|dimension|common|parameter|data|save|external|"
    r"intrinsic|equivalence)\b")


def classify(text):
    """Returns the declaration keyword if the statement is a declaration."""
    m = _DECL_RE.match(text)
    if not m:
        return None
    kw = m.group(1)
    rest = text[m.end():].lstrip()
    # "real x = ..." is not F77; but "data = 1" / "save = 2" would be assignments
    if kw in ("data", "save", "common", "parameter", "dimension") and rest.startswith("="):
        return None
    if kw.startswith(("real", "integer", "logical", "double", "character", "complex")):
        if rest.startswith("function"):
            return None
        if _find_top(text, "=") >= 0 and not kw.startswith("character"):
            return None
    return kw


def parse_exec(lines):
    """Parses the flat executable statements into nested blocks."""
    pos = [0]
    pending = []   # terminal labels of the open labelled DO loops

    def one(lab, text, origin):
        s = _parse_simple(text, origin)
        s.label = lab
        s.origin = origin
        return s

    def block(end_pred):
        """Statements until end_pred(label, text) (not consumed).  Returns
        (statements, label) where label is set when a nested DO consumed a
        terminal statement that an enclosing DO shares."""
        out = []
        while pos[0] < len(lines):
            lab, text, origin = lines[pos[0]]
            if end_pred(lab, text):
                return out, None
            pos[0] += 1
            if re.match(r"^if\s*\(", text):
                close = _match_paren(text, text.index("("))
                if text[close + 1:].strip() == "then":
                    out.append(parse_if(lab, text, origin, close))
                    continue
            m_dw = re.match(r"^do\s*(\d+)?\s*,?\s*while\s*\((.*)\)\s*$", text)
            m_do = re.match(r"^do\s*(\d+)?\s*,?\s*([a-z_]\w*)\s*=(.*)$", text)
            if m_dw or (m_do and len(_split_top(m_do.group(3))) >= 2):
                m = m_dw or m_do
                term = int(m.group(1)) if m.group(1) else None
                pending.append(term)
                body = do_body(term)
                pending.pop()
                if m_dw:
                    st = SDo(None, None, None, None, body, while_cond=parse_expr(m_dw.group(2)))
                else:
                    parts = _split_top(m_do.group(3))
                    st = SDo(m_do.group(2), parse_expr(parts[0]), parse_expr(parts[1]),
                             parse_expr(parts[2]) if len(parts) > 2 else None, body)
                st.label, st.origin = lab, origin
                out.append(st)
                if term is not None and term in pending:
                    return out, term
                continue
            out.append(one(lab, text, origin))
        return out, None

    def do_body(term):
        if term is None:
            body, _ = block(lambda l, t: re.match(r"^end\s*do$", t) is not None)
            if pos[0] >= len(lines):
                raise F77Error("DO without END DO")
            pos[0] += 1
            return body
        body, sig = block(lambda l, t: l == term)
        if sig == term:
            return body          # a nested loop consumed the shared terminal
        if pos[0] >= len(lines):
            raise F77Error(f"DO {term} without its terminal statement")
        lab, text, origin = lines[pos[0]]
        pos[0] += 1
        if re.match(r"^do\s", text) or re.match(r"^if\s*\(.*\)\s*then$", text):
            raise F77Error(f"unsupported terminal statement of DO {term}: {text!r}")
        body.append(one(lab, text, origin))
        return body

    def parse_if(lab, text, origin, close):
        cond = parse_expr(text[text.index("(") + 1:close])
        branches, else_body = [], None
        cur_cond = cond
        while True:
            body, _ = block(lambda l, t: re.match(r"^(else|end\s*if$)", t) is not None)
            if pos[0] >= len(lines):
                raise F77Error(f"IF without END IF at {origin}")
            branches.append((cur_cond, body))
            l2, t2, o2 = lines[pos[0]]
            pos[0] += 1
            if re.match(r"^else\s*if\s*\(", t2):
                c2 = _match_paren(t2, t2.index("("))
                cur_cond = parse_expr(t2[t2.index("(") + 1:c2])
                continue
            if re.match(r"^else$", t2):
                else_body, _ = block(lambda l, t: re.match(r"^end\s*if$", t) is not None)
                pos[0] += 1
            break
        st = SIf(branches, else_body)
        st.label, st.origin = lab, origin
        return st

    res, _ = block(lambda l, t: False)
    return res


def _parse_simple(text, origin):
    m = re.match(r"^if\s*\(", text)
    if m:
        close = _match_paren(text, text.index("("))
        cond = parse_expr(text[text.index("(") + 1:close])
        tail = text[close + 1:].strip()
        if re.match(r"^\d+\s*,\s*\d+\s*,\s*\d+$", tail):
            raise F77Error(f"arithmetic IF not supported at {origin}")
        inner = _parse_simple(tail, origin)
        return SIf([(cond, [inner])], None)
    m = re.match(r"^go\s*to\s*(\d+)$", text)
    if m:
        return SGoto(int(m.group(1)))
    if text == "continue":
        return SSimple("continue")
    if text == "return":
        return SSimple("return")
    if re.match(r"^stop\b", text):
        return SSimple("stop")
    if re.match(r"^(write|print|format|read|open|close|rewind|backspace|inquire|flush)\b",
                text) and _find_top(text, "=") < 0:
        return SSimple("nop")
    if re.match(r"^(write|print|format)\s*\(", text):
        return SSimple("nop")
    m = re.match(r"^call\s+([a-z_]\w*)\s*(\((.*)\))?\s*$", text)
    if m:
        args = []
        if m.group(3) is not None and m.group(3).strip():
            args = [parse_expr(a) for a in _split_top(m.group(3))]
        return SCall(m.group(1), args)
    eq = _find_top(text, "=")
    if eq > 0:
        return SAssign(parse_expr(text[:eq]), parse_expr(text[eq + 1:]))
    raise F77Error(f"cannot parse statement at {origin}: {text!r}")


# --------------------------------------------------------------- runtime --
def _w32(v):
    v &= 0xFFFFFFFF
    return v - 0x100000000 if v & 0x80000000 else v


def _idiv(a, b):
    q = abs(a) // abs(b)
    return q if (a >= 0) == (b >= 0) else -q


def _imod(a, b):
    return a - _idiv(a, b) * b


def _powi(x, m):
    """libgcc __powidf2."""
    n = -m if m < 0 else m
    y = x if n % 2 else 1.0
    while True:
        n >>= 1
        if not n:
            break
        x = x * x
        if n % 2:
            y = y * x
    return 1.0 / y if m < 0 else y


def _sqrt(x):
    return math.sqrt(x) if x >= 0 else float("nan")


def _nint(x):
    return int(math.floor(x + 0.5)) if x >= 0 else -int(math.floor(-x + 0.5))


def _sign(a, b):
    return abs(a) if b >= 0 else -abs(a)


def _fmod(a, b):
    return math.fmod(a, b)


# intrinsic name -> (python expression template, result type rule)
# rule: 'r' real, 'i' integer, 'arg' type of the first argument, 'l' logical
INTRINSICS = {
    "abs": ("abs({0})", "arg"), "dabs": ("abs({0})", "r"), "iabs": ("abs({0})", "i"),
    "sqrt": ("_sqrt({0})", "r"), "dsqrt": ("_sqrt({0})", "r"),
    "sin": ("_m.sin({0})", "r"), "dsin": ("_m.sin({0})", "r"),
    "cos": ("_m.cos({0})", "r"), "dcos": ("_m.cos({0})", "r"),
    "tan": ("_m.tan({0})", "r"), "atan": ("_m.atan({0})", "r"), "datan": ("_m.atan({0})", "r"),
    "atan2": ("_m.atan2({0},{1})", "r"), "asin": ("_m.asin({0})", "r"),
    "acos": ("_m.acos({0})", "r"), "exp": ("_m.exp({0})", "r"), "dexp": ("_m.exp({0})", "r"),
    "log": ("_m.log({0})", "r"), "alog": ("_m.log({0})", "r"), "dlog": ("_m.log({0})", "r"),
    "log10": ("_m.log10({0})", "r"), "alog10": ("_m.log10({0})", "r"),
    "sinh": ("_m.sinh({0})", "r"), "cosh": ("_m.cosh({0})", "r"), "tanh": ("_m.tanh({0})", "r"),
    "real": ("float({0})", "r"), "dble": ("float({0})", "r"), "float": ("float({0})", "r"),
    "dfloat": ("float({0})", "r"), "sngl": ("float({0})", "r"),
    "int": ("int({0})", "i"), "ifix": ("int({0})", "i"), "idint": ("int({0})", "i"),
    "nint": ("_nint({0})", "i"), "idnint": ("_nint({0})", "i"),
    "sign": ("_sign({0},{1})", "arg"), "dsign": ("_sign({0},{1})", "r"),
    "isign": ("_sign({0},{1})", "i"),
}


def _implicit_default():
    return {chr(c): ("i4" if "i" <= chr(c) <= "n" else "r8") for c in range(ord("a"), ord("z") + 1)}


class Sym:
    def __init__(self, name):
        self.name = name
        self.type = None
        self.dims = None          # list of (lo_expr, hi_expr|None)
        self.kind = "local"       # local, dummy, common, param
        self.common = None        # (block, index)
        self.value = None         # parameter value
        self.static = False
        self.data = None          # list of initial values
        self.external = False
        self.char_len = None


class F77:
    """Loads Fortran sources and runs their subroutines and functions."""

    def __init__(self, files, include_dirs, defines=(), overrides=None, externals=None):
        self.units = {}
        for f in files:
            for u in split_units(read_statements(f, include_dirs, defines, overrides)):
                self.units[u.name] = u
        self.externals = dict(externals or {})
        self.commons = {}       # block -> list of storage lists
        self.common_layout = {}  # block -> list of sizes
        self.compiled = {}
        self.static = {}
        self.trace = None

    # ------------------------------------------------------------ public --
    def common(self, block):
        """Storage lists of a COMMON block (in declaration order)."""
        return self.commons[block]

    def call(self, name, *args):
        """Calls a routine with Ref / list / scalar arguments."""
        fn = self.routine(name)
        refs = []
        for a in args:
            if isinstance(a, Ref):
                refs.append(a)
            elif isinstance(a, list):
                refs.append(Ref(a, 0))
            else:
                refs.append(Ref([a], 0))
        return fn(*refs)

    def routine(self, name):
        if name in self.compiled:
            return self.compiled[name]
        if name in self.units:
            fn = self._compile(self.units[name])
            self.compiled[name] = fn
            return fn
        if name in self.externals:
            return self.externals[name]
        raise F77Error(f"routine {name} is neither in the sources nor an external")

    def ensure_common(self, block):
        """Declares a COMMON block from the first unit that names it (without
        running anything)."""
        if block not in self.commons:
            for u in self.units.values():
                if any(text.startswith("common") and f"/{block}/" in text.replace(" ", "")
                       for _, text, _ in u.body):
                    self._analyse(u)
                    break
        if block not in self.commons:
            raise F77Error(f"no unit declares COMMON /{block}/")
        return self.commons[block]

    # -------------------------------------------------------- analysis --
    def _analyse(self, u):
        if getattr(u, "syms", None) is not None:
            return
        implicit = _implicit_default()
        syms = {}

        def sym(n):
            if n not in syms:
                syms[n] = Sym(n)
            return syms[n]

        for a in u.args:
            s = sym(a)
            s.kind = "dummy"
        exec_lines = []
        decls = []
        for lab, text, origin in u.body:
            kw = classify(text)
            if kw is None:
                exec_lines.append((lab, text, origin))
            else:
                decls.append((kw, text, origin))
        u.exec_lines = exec_lines
        commons = []   # (block, [names])
        equivs = []    # (a, b, origin)
        # first pass: implicit, parameters in order with types
        for kw, text, origin in decls:
            if kw == "implicit":
                rest = text[len("implicit"):].strip()
                if rest == "none":
                    implicit = {}
                    continue
                for m in re.finditer(r"(double precision|real\*8|real\*4|real|integer\*8|"
                                     r"integer|logical)\s*\(([^)]*)\)", rest):
                    t = dict(TYPE_WORDS)[m.group(1)]
                    for rng in m.group(2).split(","):
                        rng = rng.strip()
                        if "-" in rng:
                            a, b = [x.strip() for x in rng.split("-")]
                        else:
                            a = b = rng
                        for c in range(ord(a), ord(b) + 1):
                            implicit[chr(c)] = t
        u.implicit = implicit

        def type_of(s):
            if s.type:
                return s.type
            return implicit.get(s.name[0], "r8")

        for kw, text, origin in decls:
            if kw == "implicit":
                continue
            if kw in ("save",):
                rest = text[4:].strip()
                for n in [x.strip() for x in rest.split(",") if x.strip()]:
                    if n.startswith("/"):
                        continue
                    sym(n).static = True
                if not rest:
                    u.save_all = True
                continue
            if kw in ("external", "intrinsic"):
                for n in text[len(kw):].split(","):
                    if n.strip():
                        sym(n.strip()).external = kw == "external"
                continue
            if kw == "equivalence":
                # whole-array pairs only: (a, b) makes b share a's storage
                for m in re.finditer(r"\(\s*([a-z_]\w*)\s*,\s*([a-z_]\w*)\s*\)", text):
                    equivs.append((m.group(1), m.group(2), origin))
                if not re.fullmatch(r"equivalence\s*(\(\s*[a-z_]\w*\s*,\s*[a-z_]\w*\s*\)"
                                    r"\s*,?\s*)+", text):
                    raise F77Error(f"only whole-array EQUIVALENCE pairs are supported ({origin})")
                continue
            if kw == "parameter":
                inner = text[text.index("(") + 1:text.rindex(")")]
                for item in _split_top(inner):
                    n, e = item.split("=", 1)
                    s = sym(n.strip())
                    s.kind = "param"
                    s.value = self._const_eval(parse_expr(e), syms, implicit)
                    t = type_of(s)
                    s.value = float(s.value) if t in ("r8", "r4") else (
                        int(s.value) if t in ("i4", "i8") else s.value)
                continue
            if kw == "common":
                rest = text[len("common"):].strip()
                for m in re.finditer(r"/\s*([a-z_]\w*)?\s*/([^/]*)", rest):
                    block = m.group(1) or "_blank_"
                    names = []
                    for item in _split_top(m.group(2).strip().rstrip(",")):
                        if not item:
                            continue
                        mm = re.match(r"^([a-z_]\w*)\s*(\((.*)\))?$", item)
                        s = sym(mm.group(1))
                        s.kind = "common"
                        if mm.group(3):
                            s.dims = self._dims(mm.group(3))
                        names.append(s.name)
                    commons.append((block, names))
                continue
            if kw == "data":
                rest = text[4:].strip()
                for m in re.finditer(r"([^/]+)/([^/]*)/\s*,?", rest):
                    names = _split_top(m.group(1).strip().strip(","))
                    vals = []
                    for v in _split_top(m.group(2)):
                        if "*" in v and re.match(r"^\d+\s*\*", v):
                            cnt, vv = v.split("*", 1)
                            vals.extend([self._const_eval(parse_expr(vv), syms, implicit)] *
                                        int(cnt))
                        else:
                            vals.append(self._const_eval(parse_expr(v), syms, implicit))
                    k = 0
                    for n in names:
                        s = sym(n.strip())
                        s.static = True
                        if s.dims:
                            size = self._static_size(s, syms, implicit)
                            s.data = vals[k:k + size]
                            k += size
                        else:
                            s.data = [vals[k]]
                            k += 1
                continue
            # type declarations and DIMENSION
            t = None
            rest = text
            if kw != "dimension":
                for word, tt in TYPE_WORDS:
                    if text.startswith(word):
                        t = tt
                        rest = text[len(word):]
                        break
                if t == "c":
                    m = re.match(r"^\*\s*(\d+|\(\*\))", rest)
                    if m:
                        rest = rest[m.end():]
            else:
                rest = text[len("dimension"):]
            for item in _split_top(rest.strip()):
                if not item:
                    continue
                mm = re.match(r"^([a-z_]\w*)\s*(\*\s*\d+)?\s*(\((.*)\))?(\s*\*\s*\d+)?$", item)
                if not mm:
                    raise F77Error(f"cannot parse declaration item {item!r} at {origin}")
                s = sym(mm.group(1))
                if t:
                    s.type = t
                if mm.group(4):
                    s.dims = self._dims(mm.group(4))
        for n, s in syms.items():
            if s.kind != "param":
                s.type = type_of(s)
        if u.kind == "function":
            rs = sym(u.name)
            if u.rtype:
                rs.type = u.rtype
            rs.type = rs.type or implicit.get(u.name[0], "r8")
            rs.kind = "result"
        u.syms = syms
        # COMMON layout (storage association by position)
        for block, names in commons:
            sizes = []
            for n in names:
                s = syms[n]
                sizes.append(self._static_size(s, syms, implicit) if s.dims else 1)
            if block not in self.commons:
                self.common_layout[block] = sizes
                store = []
                for n, sz in zip(names, sizes):
                    t = syms[n].type
                    zero = 0.0 if t in ("r8", "r4") else (False if t == "l" else
                                                          ("" if t == "c" else 0))
                    store.append([zero] * sz)
                self.commons[block] = store
            else:
                old = self.common_layout[block]
                if old != sizes:
                    raise F77Error(f"COMMON /{block}/ declared with different layouts in "
                                   f"{u.name}: {sizes} vs {old}")
            for k, n in enumerate(names):
                syms[n].common = (block, k)
        for a, b, origin in equivs:
            sa, sb = syms.get(a), syms.get(b)
            if sa is None or sb is None:
                raise F77Error(f"EQUIVALENCE of undeclared names ({origin})")
            if sb.common is not None and sa.common is None:
                sa, sb = sb, sa
            if sa.common is not None:
                sb.kind = "common"
                sb.common = sa.common
            else:
                sb.alias = a
        u.tree = parse_exec(u.exec_lines)

    def _dims(self, text):
        out = []
        for d in _split_top(text):
            if d == "*":
                out.append((Num(1), None))
            elif ":" in d:
                a, b = d.split(":", 1)
                out.append((parse_expr(a), None if b.strip() == "*" else parse_expr(b)))
            else:
                out.append((Num(1), parse_expr(d)))
        return out

    def _const_eval(self, e, syms, implicit):
        if isinstance(e, Num):
            return e.v
        if isinstance(e, Str):
            return e.v
        if isinstance(e, Bool):
            return e.v
        if isinstance(e, Name):
            s = syms.get(e.name)
            if s is None or s.kind != "param":
                raise F77Error(f"{e.name} is not a constant")
            return s.value
        if isinstance(e, UnOp):
            v = self._const_eval(e.a, syms, implicit)
            return -v if e.op == "-" else (v if e.op == "+" else (not v))
        if isinstance(e, BinOp):
            a = self._const_eval(e.a, syms, implicit)
            b = self._const_eval(e.b, syms, implicit)
            if e.op == "+":
                return a + b
            if e.op == "-":
                return a - b
            if e.op == "*":
                return _w32(a * b) if isinstance(a, int) and isinstance(b, int) else a * b
            if e.op == "/":
                return _idiv(a, b) if isinstance(a, int) and isinstance(b, int) else a / b
            if e.op == "**":
                if isinstance(a, int) and isinstance(b, int):
                    return a ** b
                if isinstance(b, int):
                    return _powi(float(a), b)
                return float(a) ** b
        if isinstance(e, Apply):
            if e.name in ("max", "min"):
                vals = [self._const_eval(x, syms, implicit) for x in e.args]
                return max(vals) if e.name == "max" else min(vals)
        raise F77Error("unsupported constant expression")

    def _static_size(self, s, syms, implicit):
        size = 1
        for lo, hi in s.dims:
            if hi is None:
                raise F77Error(f"assumed-size array {s.name} cannot be static")
            size *= self._const_eval(hi, syms, implicit) - self._const_eval(lo, syms, implicit) + 1
        return size

    # ------------------------------------------------------------ codegen --
    def _compile(self, u):
        self._analyse(u)
        g = _Gen(self, u)
        src = g.generate()
        env = {"_m": math, "_w32": _w32, "_idiv": _idiv, "_imod": _imod, "_powi": _powi,
               "_sqrt": _sqrt, "_nint": _nint, "_sign": _sign, "_fmod": _fmod, "Ref": Ref,
               "_Goto": _Goto, "_Return": _Return, "_Stop": _Stop, "_rt": self,
               "_C": self.commons, "_S": self.static.setdefault(u.name, {})}
        u.pysrc = src
        try:
            exec(compile(src, f"<f77:{u.name}>", "exec"), env)
        except SyntaxError as ex:
            raise F77Error(f"generated code for {u.name} does not compile: {ex}\n{src}")
        return env["U_" + u.name]


class _Gen:
    """Python source of one program unit."""

    def __init__(self, rt, u):
        self.rt, self.u, self.syms = rt, u, u.syms
        self.lines = []
        self.tmp = 0
        self.assigned = set()
        self.goto_targets = set()
        self.auto_arrays = []
        self._scan(u.tree)

    def _scan(self, body):
        for s in body:
            if isinstance(s, SAssign):
                t = s.target
                self.assigned.add(t.name if isinstance(t, (Name, Apply)) else None)
            elif isinstance(s, SCall):
                for a in s.args:
                    if isinstance(a, (Name, Apply)):
                        self.assigned.add(a.name)
            elif isinstance(s, SIf):
                for c, b in s.branches:
                    self._scan(b)
                if s.else_body:
                    self._scan(s.else_body)
            elif isinstance(s, SDo):
                if s.var:
                    self.assigned.add(s.var)
                self._scan(s.body)
            elif isinstance(s, SGoto):
                self.goto_targets.add(s.target)

    def _const_dims(self, s):
        try:
            self.rt._static_size(s, self.syms, self.u.implicit)
            return True
        except F77Error:
            return False

    def new(self):
        self.tmp += 1
        return f"_t{self.tmp}"

    def emit(self, ind, text):
        self.lines.append("    " * ind + text)

    # --- symbols
    def sym(self, name):
        s = self.syms.get(name)
        if s is None:
            s = Sym(name)
            s.type = self.u.implicit.get(name[0], "r8")
            self.syms[name] = s
        return s

    def is_array(self, name):
        s = self.syms.get(name)
        return s is not None and s.dims is not None

    def is_function(self, name):
        if self.is_array(name):
            return False
        return True

    def fn_type(self, name, args_types):
        if name in INTRINSICS:
            rule = INTRINSICS[name][1]
            if rule == "arg":
                return args_types[0]
            return {"r": "r8", "i": "i4", "l": "l"}[rule]
        if name in ("max", "min", "amax1", "amin1", "dmax1", "dmin1", "max0", "min0"):
            if name in ("amax1", "amin1", "dmax1", "dmin1"):
                return "r8"
            if name in ("max0", "min0"):
                return "i4"
            return "r8" if "r8" in args_types else "i4"
        if name in ("mod", "amod", "dmod"):
            return "r8" if (name != "mod" or "r8" in args_types) else "i4"
        if name in self.rt.units:
            fu = self.rt.units[name]
            self.rt._analyse(fu)
            return fu.syms[fu.name].type
        s = self.syms.get(name)
        if s is not None and s.type:
            return s.type
        return self.u.implicit.get(name[0], "r8")

    # --- expressions: returns (python source, type)
    def expr(self, e):
        if isinstance(e, Num):
            if isinstance(e.v, int):
                return str(e.v), "i4"
            return repr(float(e.v)), "r8"
        if isinstance(e, Str):
            return repr(e.v), "c"
        if isinstance(e, Bool):
            return ("True" if e.v else "False"), "l"
        if isinstance(e, Name):
            return self.scalar_ref(e.name)
        if isinstance(e, Apply):
            if self.is_array(e.name):
                return self.elem_ref(e.name, e.args), self.sym(e.name).type
            return self.fcall(e.name, e.args)
        if isinstance(e, UnOp):
            a, t = self.expr(e.a)
            if e.op == "-":
                return f"(-{a})", t
            if e.op == "+":
                return a, t
            return f"(not {a})", "l"
        if isinstance(e, BinOp):
            a, ta = self.expr(e.a)
            b, tb = self.expr(e.b)
            op = e.op
            if op in ("and", "or"):
                return f"({a} {op} {b})", "l"
            if op == "eqv":
                return f"({a} == {b})", "l"
            if op == "neqv":
                return f"({a} != {b})", "l"
            if op in ("==", "!=", "<", "<=", ">", ">="):
                return f"({a} {op} {b})", "l"
            if op == "//":
                return f"({a} + {b})", "c"
            isint = ta in ("i4", "i8") and tb in ("i4", "i8")
            if op == "**":
                if isint:
                    return f"({a} ** {b})", ta
                if tb in ("i4", "i8"):
                    return f"_powi(float({a}), {b})", "r8"
                return f"(float({a}) ** {b})", "r8"
            if isint:
                t = "i8" if "i8" in (ta, tb) else "i4"
                if op == "/":
                    return f"_idiv({a}, {b})", t
                if op == "*" and t == "i4":
                    return f"_w32({a} * {b})", t
                return f"({a} {op} {b})", t
            return f"({a} {op} {b})", "r8"
        raise F77Error("bad expression")

    def scalar_ref(self, name):
        s = self.sym(name)
        if s.kind == "param":
            v = s.value
            if isinstance(v, float):
                return repr(v), "r8"
            if isinstance(v, bool):
                return repr(v), "l"
            if isinstance(v, int):
                return str(v), s.type or "i4"
            return repr(v), "c"
        if s.dims is not None:
            raise F77Error(f"array {name} used as a scalar in {self.u.name}")
        if s.kind == "common":
            return f"cm_{name}[0]", s.type
        if s.static:
            return f"st_{name}[0]", s.type
        if s.kind == "result":
            return "_res", s.type
        if name not in self.syms or (s.kind == "local" and s.type is None):
            pass
        return f"v_{name}", s.type

    def elem_index(self, name, args):
        s = self.sym(name)
        if len(args) != len(s.dims):
            raise F77Error(f"{name}: {len(args)} subscripts for rank {len(s.dims)} "
                           f"in {self.u.name}")
        terms = []
        for k, a in enumerate(args):
            src, t = self.expr(a)
            if k == 0:
                terms.append(f"{src}")
            else:
                terms.append(f"a_{name}_s{k} * ({src})")
        return f"a_{name}_o + " + " + ".join(terms)

    def elem_ref(self, name, args):
        return f"a_{name}_b[{self.elem_index(name, args)}]"

    def fcall(self, name, args):
        types = []
        srcs = []
        for a in args:
            if isinstance(a, Name) and self.is_array(a.name):
                srcs.append(None)
                types.append(self.sym(a.name).type)
                continue
            sv, tv = self.expr(a)
            srcs.append(sv)
            types.append(tv)
        if name in INTRINSICS and name not in self.rt.units:
            tmpl, _ = INTRINSICS[name]
            rt = self.fn_type(name, types)
            return tmpl.format(*srcs), rt
        if name in ("max", "min", "amax1", "amin1", "dmax1", "dmin1", "max0", "min0") \
                and name not in self.rt.units:
            rt = self.fn_type(name, types)
            f = "max" if "max" in name else "min"
            if rt == "r8":
                return f"float({f}({', '.join(srcs)}))", "r8"
            return f"{f}({', '.join(srcs)})", rt
        if name in ("mod", "amod", "dmod") and name not in self.rt.units:
            rt = self.fn_type(name, types)
            if rt == "r8":
                return f"_fmod({srcs[0]}, {srcs[1]})", "r8"
            return f"_imod({srcs[0]}, {srcs[1]})", "i4"
        # user function
        refs = [self.actual(a) for a in args]
        rt = self.fn_type(name, types)
        return f"_rt.routine({name!r})({', '.join(refs)})", rt

    def actual(self, a):
        """Source of a Ref for an actual argument (expression context)."""
        if isinstance(a, Name):
            s = self.sym(a.name)
            if s.dims is not None:
                return f"Ref(a_{a.name}_b, a_{a.name}_o0)"
            if s.kind == "common":
                return f"Ref(cm_{a.name}, 0)"
            if s.static and s.kind != "param":
                return f"Ref(st_{a.name}, 0)"
        if isinstance(a, Apply) and self.is_array(a.name):
            return f"Ref(a_{a.name}_b, {self.elem_index(a.name, a.args)})"
        src, t = self.expr(a)
        return f"Ref([{src}], 0)"

    # --- statements
    def conv(self, src, st, tt):
        if tt in ("r8", "r4") and st in ("i4", "i8"):
            return f"float({src})"
        if tt in ("i4", "i8") and st in ("r8", "r4"):
            return f"int({src})"
        return src

    def assign_target(self, t):
        if isinstance(t, Name):
            dst, tt = self.scalar_ref(t.name)
            return dst, tt
        if isinstance(t, Apply):
            if not self.is_array(t.name):
                raise F77Error(f"assignment to non-array {t.name}(...) in {self.u.name}")
            return self.elem_ref(t.name, t.args), self.sym(t.name).type
        raise F77Error("bad assignment target")

    def stmts(self, body, ind):
        if not body:
            self.emit(ind, "pass")
            return
        labels = {s.label for s in body if not isinstance(s, tuple) and s.label is not None}
        targets = labels & self.goto_targets
        if targets:
            # a block with goto targets: a resumable statement sequence
            pc = self.new()
            self.emit(ind, f"{pc} = 0")
            self.emit(ind, "while True:")
            self.emit(ind + 1, "try:")
            idx = {}
            for k, s in enumerate(body):
                if s.label in targets:
                    idx[s.label] = k
                self.emit(ind + 2, f"if {pc} <= {k}:")
                self.stmt(s, ind + 3)
            self.emit(ind + 2, "break")
            self.emit(ind + 1, "except _Goto as _g:")
            for lab, k in idx.items():
                self.emit(ind + 2, f"if _g.label == {lab}:")
                self.emit(ind + 3, f"{pc} = {k}")
                self.emit(ind + 3, "continue")
            self.emit(ind + 2, "raise")
            return
        for s in body:
            self.stmt(s, ind)

    def stmt(self, s, ind):
        if isinstance(s, SAssign):
            src, st = self.expr(s.expr)
            dst, tt = self.assign_target(s.target)
            self.emit(ind, f"{dst} = {self.conv(src, st, tt)}")
        elif isinstance(s, SCall):
            self.call(s, ind)
        elif isinstance(s, SIf):
            first = True
            for cond, body in s.branches:
                c, _ = self.expr(cond)
                self.emit(ind, f"{'if' if first else 'elif'} {c}:")
                self.stmts(body, ind + 1)
                first = False
            if s.else_body is not None:
                self.emit(ind, "else:")
                self.stmts(s.else_body, ind + 1)
        elif isinstance(s, SDo):
            if s.while_cond is not None:
                c, _ = self.expr(s.while_cond)
                self.emit(ind, f"while {c}:")
                self.stmts(s.body, ind + 1)
                return
            v, vt = self.scalar_ref(s.var)
            a, _ = self.expr(s.start)
            b, _ = self.expr(s.end)
            if s.step is not None:
                c, _ = self.expr(s.step)
            else:
                c = "1"
            ta, tb, tc, tn = self.new(), self.new(), self.new(), self.new()
            self.emit(ind, f"{ta} = {a}; {tb} = {b}; {tc} = {c}")
            self.emit(ind, f"{tn} = ({tb} - {ta} + {tc}) // {tc}")
            it = self.new()
            self.emit(ind, f"for {it} in range({ta}, {ta} + max({tn}, 0) * {tc}, {tc}):")
            self.emit(ind + 1, f"{v} = {it}")
            self.stmts(s.body, ind + 1)
            self.emit(ind, f"{v} = {ta} + max({tn}, 0) * {tc}")
        elif isinstance(s, SGoto):
            self.emit(ind, f"raise _Goto({s.target})")
        elif isinstance(s, SSimple):
            if s.kind == "return":
                self.emit(ind, "raise _Return()")
            elif s.kind == "stop":
                self.emit(ind, "raise _Stop()")
            else:
                self.emit(ind, "pass")
        else:
            raise F77Error(f"unknown statement {s!r}")

    def call(self, s, ind):
        post = []
        refs = []
        for a in s.args:
            if isinstance(a, Name):
                sy = self.sym(a.name)
                if sy.dims is None and sy.kind == "dummy":
                    # pass the caller's own reference through (an undeclared
                    # dummy may be an array the unit only hands on)
                    self.emit(ind, f"r_{a.name}.b[r_{a.name}.o] = v_{a.name}")
                    refs.append(f"r_{a.name}")
                    post.append(f"v_{a.name} = r_{a.name}.b[r_{a.name}.o]")
                    continue
                if sy.dims is None and sy.kind not in ("common", "param") and not sy.static:
                    t = self.new()
                    src, _ = self.scalar_ref(a.name)
                    self.emit(ind, f"{t} = Ref([{src}], 0)")
                    refs.append(t)
                    post.append(f"{src} = {t}.b[0]")
                    continue
            refs.append(self.actual(a))
        self.emit(ind, f"_rt.routine({s.name!r})({', '.join(refs)})")
        for p in post:
            self.emit(ind, p)

    def generate(self):
        u = self.u
        self.emit(0, f"def U_{u.name}({', '.join('r_' + a for a in u.args)}):")
        ind = 1
        # COMMON storage
        for n, s in self.syms.items():
            if s.kind == "common":
                blk, k = s.common
                if s.dims is not None:
                    self.emit(ind, f"a_{n}_b = _C[{blk!r}][{k}]")
                else:
                    self.emit(ind, f"cm_{n} = _C[{blk!r}][{k}]")
        # static locals (SAVE / DATA) and local arrays (static, as gfortran
        # places large local arrays).  Local arrays get 4x slack: the
        # reference writes past one of them (proxy_setupds' glo_num is sized
        # for lx1 points per direction, h1mg_setup_dssum asks it for lx1+2),
        # which in the compiled program lands in memory nothing else uses.
        for n, s in self.syms.items():
            if s.kind == "local" and s.dims is not None and not s.static and \
                    not self._const_dims(s):
                # automatic array (bounds from dummies or COMMON), fresh per call
                ext = []
                for lo, hi in s.dims:
                    los, _ = self.expr(lo)
                    his, _ = self.expr(hi)
                    ext.append(f"(({his}) - ({los}) + 1)")
                zero = "0.0" if s.type in ("r8", "r4") else "0"
                self.auto_arrays.append((n, f"[{zero}] * ({' * '.join(ext)})"))
                continue
            if s.kind in ("local",) and (s.static or s.dims is not None):
                size = self.rt._static_size(s, self.syms, u.implicit) if s.dims else 1
                if s.dims is not None:
                    size *= 4
                zero = "0.0" if s.type in ("r8", "r4") else ("False" if s.type == "l" else
                                                             ("''" if s.type == "c" else "0"))
                init = repr(list(s.data)) if s.data else f"[{zero}] * {size}"
                if s.data and len(s.data) < size:
                    init = f"{init} + [{zero}] * {size - len(s.data)}"
                name = f"a_{n}_b" if s.dims is not None else f"st_{n}"
                key = getattr(s, "alias", None) or n
                self.emit(ind, f"if {key!r} not in _S: _S[{key!r}] = {init}")
                self.emit(ind, f"{name} = _S[{key!r}]")
                if s.dims is None:
                    s.static = True
        # dummies
        for a in u.args:
            s = self.syms[a]
            if s.dims is not None:
                self.emit(ind, f"a_{a}_b = r_{a}.b")
            else:
                self.emit(ind, f"v_{a} = r_{a}.b[r_{a}.o]")
        for n, init in self.auto_arrays:
            self.emit(ind, f"a_{n}_b = {init}")
        # array offsets and strides (dummy bounds may use dummy scalars and commons)
        for n, s in self.syms.items():
            if s.dims is None or s.kind == "param":
                continue
            base = f"r_{n}.o" if s.kind == "dummy" else "0"
            self.emit(ind, f"a_{n}_o0 = {base}")
            stride = "1"
            off_terms = []
            for k, (lo, hi) in enumerate(s.dims):
                los, _ = self.expr(lo)
                if k > 0:
                    self.emit(ind, f"a_{n}_s{k} = {stride}")
                    off_terms.append(f"a_{n}_s{k} * ({los})")
                else:
                    off_terms.append(f"({los})")
                if hi is not None:
                    his, _ = self.expr(hi)
                    stride = f"(a_{n}_s{k} * (({his}) - ({los}) + 1))" if k > 0 else \
                        f"(({his}) - ({los}) + 1)"
                else:
                    stride = "0"
            self.emit(ind, f"a_{n}_o = a_{n}_o0 - ({' + '.join(off_terms)})")
        # DATA-initialised scalars that are not static were made static above
        if u.kind == "function":
            z = "0.0" if self.syms[u.name].type in ("r8", "r4") else "0"
            self.emit(ind, f"_res = {z}")
        # scalar locals default
        self._defaulted = set()
        for n, s in self.syms.items():
            if s.kind == "local" and s.dims is None and not s.static and not s.external:
                z = "0.0" if s.type in ("r8", "r4") else ("False" if s.type == "l" else
                                                          ("''" if s.type == "c" else "0"))
                self.emit(ind, f"v_{n} = {z}")
                self._defaulted.add(n)
        # the body first (it registers implicitly typed scalars), then their
        # defaults ahead of it
        head = self.lines
        self.lines = []
        self.stmts(u.tree, ind + 1)
        body = self.lines
        self.lines = head
        for n, s in self.syms.items():
            if n in self._defaulted or s.kind != "local" or s.dims is not None or s.static \
                    or s.external:
                continue
            z = "0.0" if s.type in ("r8", "r4") else ("False" if s.type == "l" else
                                                      ("''" if s.type == "c" else "0"))
            self.emit(ind, f"v_{n} = {z}")
        self.emit(ind, "try:")
        self.lines.extend(body)
        self.emit(ind, "except _Return:")
        self.emit(ind + 1, "pass")
        # copy out dummy scalars that may have changed
        for a in u.args:
            s = self.syms[a]
            if s.dims is None and a in self.assigned:
                self.emit(ind, f"r_{a}.b[r_{a}.o] = v_{a}")
        if u.kind == "function":
            self.emit(ind, "return _res")
        return "\n".join(self.lines) + "\n"
