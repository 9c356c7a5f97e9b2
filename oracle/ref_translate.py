"""Test infrastructure only: translate the reference's Fortran routines into C.

No Fortran compiler is available, so to run the
reference's own code (the parity pin for the C++ restatement in
broadcast_oracle.hpp) its source files are translated mechanically into C by
this script and compiled with gcc (oracle/ref_build.py).  The translator
covers the subset of Fortran 90 those files use: subroutines with explicit
shape arrays and arbitrary lower bounds, integer/real(8)/character scalars,
DO loops, IF blocks, whole-array and section assignments, the intrinsics
SQRT ABS TANH MAX MIN SIGN FLOAT INT MOD REAL, ** powers, and the
PUSH/POP calls of Tapenade's static taping (a private LIFO stack).

Semantics follow the reference's build flags (srcfv/compile_rhs.py:25-29):
default reals are 8-byte (-r8 / -fdefault-real-8), so every real literal is
double.  The generated C goes to oracle/_ref/ only and is never committed.
"""
import re

KEYWORDS = {"and", "or", "not", "eq", "ne", "lt", "le", "gt", "ge", "true", "false"}


class TranslateError(Exception):
    pass


# ---------------------------------------------------------------------------
# source preparation
def _strip_comment(line):
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


def logical_lines(text):
    """Comment-free statements with continuations joined and ';' split."""
    raw = [_strip_comment(l).rstrip() for l in text.splitlines()]
    stmts, buf = [], ""
    for l in raw:
        s = l.strip()
        if not s:
            continue
        if s.startswith("#"):
            continue
        if buf:
            if s.startswith("&"):
                s = s[1:]
            buf += " " + s.strip()
        else:
            buf = s
        if buf.endswith("&"):
            buf = buf[:-1]
            continue
        for part in _split_semicolons(buf):
            if part.strip():
                stmts.append(part.strip())
        buf = ""
    return stmts


def _split_semicolons(s):
    parts, cur, q = [], [], None
    for ch in s:
        if q:
            cur.append(ch)
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
            cur.append(ch)
        elif ch == ";":
            parts.append("".join(cur))
            cur = []
        else:
            cur.append(ch)
    parts.append("".join(cur))
    return parts


# ---------------------------------------------------------------------------
# expressions
TOKEN = re.compile(r"""
    (?P<ws>\s+)
  | (?P<num>(\d+\.\d*|\.\d+|\d+)([dDeE][+-]?\d+)?(_\d+)?)
  | (?P<dotop>\.(and|or|not|eq|ne|lt|le|gt|ge|true|false)\.)
  | (?P<str>'[^']*'|"[^"]*")
  | (?P<name>[A-Za-z_][A-Za-z_0-9]*)
  | (?P<op>\*\*|==|/=|<=|>=|=>|[-+*/(),:<>=])
""", re.X | re.I)


def tokenize(s):
    toks, pos = [], 0
    while pos < len(s):
        m = TOKEN.match(s, pos)
        if not m:
            raise TranslateError("cannot tokenize %r at %d" % (s, pos))
        pos = m.end()
        kind = m.lastgroup
        if kind == "ws":
            continue
        txt = m.group(kind)
        if kind == "dotop":
            toks.append(("op", "." + m.group(kind)[1:-1].lower() + "."))
        elif kind == "name":
            toks.append(("name", txt.lower()))
        elif kind == "num":
            toks.append(("num", txt))
        else:
            toks.append((kind, txt))
    return toks


class Expr:
    def __init__(self, code, typ):
        self.code, self.typ = code, typ  # typ in 'int', 'real', 'bool', 'str'


class ExprParser:
    """Recursive descent over Fortran expressions producing C."""

    def __init__(self, toks, sub):
        self.t, self.i, self.sub = toks, 0, sub

    def peek(self, k=0):
        return self.t[self.i + k] if self.i + k < len(self.t) else (None, None)

    def take(self, val=None):
        tok = self.peek()
        if val is not None and tok[1] != val:
            raise TranslateError("expected %r got %r" % (val, tok))
        self.i += 1
        return tok

    def parse(self):
        e = self.eqv()
        return e

    def eqv(self):
        return self.orx()

    def orx(self):
        a = self.andx()
        while self.peek()[1] == ".or.":
            self.take()
            b = self.andx()
            a = Expr("(%s || %s)" % (a.code, b.code), "bool")
        return a

    def andx(self):
        a = self.notx()
        while self.peek()[1] == ".and.":
            self.take()
            b = self.notx()
            a = Expr("(%s && %s)" % (a.code, b.code), "bool")
        return a

    def notx(self):
        if self.peek()[1] == ".not.":
            self.take()
            a = self.notx()
            return Expr("(!%s)" % a.code, "bool")
        return self.rel()

    REL = {".eq.": "==", "==": "==", ".ne.": "!=", "/=": "!=", ".lt.": "<", "<": "<", ".le.": "<=", "<=": "<=",
           ".gt.": ">", ">": ">", ".ge.": ">=", ">=": ">="}

    def rel(self):
        a = self.add()
        op = self.peek()[1]
        if op in self.REL:
            self.take()
            b = self.add()
            if a.typ == "str" or b.typ == "str":
                s = b if b.typ == "str" and b.code.startswith('"') else a
                o = a if s is b else b
                n = len(s.code) - 2
                cmp = "(strncmp(%s, %s, %d) %s 0)" % (o.code, s.code, n, self.REL[op])
                return Expr(cmp, "bool")
            return Expr("(%s %s %s)" % (a.code, self.REL[op], b.code), "bool")
        return a

    def add(self):
        if self.peek()[1] in ("+", "-"):
            op = self.take()[1]
            a = self.mul()
            a = Expr("(%s%s)" % (op, a.code), a.typ)
        else:
            a = self.mul()
        while self.peek()[1] in ("+", "-"):
            op = self.take()[1]
            b = self.mul()
            a = Expr("(%s %s %s)" % (a.code, op, b.code), _arith(a, b))
        return a

    def mul(self):
        a = self.power()
        while self.peek()[1] in ("*", "/"):
            op = self.take()[1]
            b = self.power()
            a = Expr("(%s %s %s)" % (a.code, op, b.code), _arith(a, b))
        return a

    def power(self):
        a = self.unary()
        if self.peek()[1] == "**":
            self.take()
            if self.peek()[1] in ("+", "-"):
                sign = self.take()[1]
                b = self.power()
                b = Expr("(%s%s)" % (sign, b.code), b.typ)
            else:
                b = self.power()  # right associative
            if b.typ == "int" and re.fullmatch(r"\(?\d+\)?", b.code):
                n = int(b.code.strip("()"))
                if a.typ == "int":
                    return Expr("f_ipowi(%s, %d)" % (a.code, n), "int")
                if n == 2:
                    return Expr("f_sq(%s)" % a.code, "real")
                return Expr("f_powi(%s, %d)" % (a.code, n), "real")
            return Expr("pow((double)(%s), (double)(%s))" % (a.code, b.code), "real")
        return a

    def unary(self):
        tok = self.peek()
        if tok[1] in ("+", "-"):
            op = self.take()[1]
            a = self.unary()
            return Expr("(%s%s)" % (op, a.code), a.typ)
        return self.primary()

    def primary(self):
        kind, txt = self.take()
        if kind == "num":
            return _number(txt)
        if kind == "str":
            return Expr('"%s"' % txt[1:-1], "str")
        if kind == "op" and txt in (".true.", ".false."):
            return Expr("1" if txt == ".true." else "0", "bool")
        if kind == "op" and txt == "(":
            e = self.parse()
            self.take(")")
            return Expr("(%s)" % e.code, e.typ)
        if kind == "name":
            if self.peek()[1] == "(":
                self.take("(")
                args = []
                if self.peek()[1] != ")":
                    args.append(self.arg())
                    while self.peek()[1] == ",":
                        self.take()
                        args.append(self.arg())
                self.take(")")
                return self.sub.ref(txt, args)
            return self.sub.ref(txt, None)
        raise TranslateError("unexpected token %r" % ((kind, txt),))

    def arg(self):
        if self.peek()[1] == ":" or (self.peek()[1] is not None and self.peek(1)[1] == ":"
                                     and self.peek()[0] in ("num", "name")):
            # section a:b or :
            lo = hi = None
            if self.peek()[1] != ":":
                lo = self.add()
            self.take(":")
            if self.peek()[1] not in (",", ")"):
                hi = self.add()
            return ("section", lo, hi)
        return self.parse()


def _arith(a, b):
    return "int" if a.typ == "int" and b.typ == "int" else "real"


def _number(txt):
    t = txt.lower()
    t = re.sub(r"_\d+$", "", t)
    if re.fullmatch(r"\d+", t):
        return Expr(t, "int")
    t = t.replace("d", "e")
    if t.startswith("."):
        t = "0" + t
    m = re.fullmatch(r"(\d+)\.?(\d*)(e[+-]?\d+)?", t)
    if not m:
        raise TranslateError("bad number %r" % txt)
    mant = m.group(1) + "." + (m.group(2) or "0")
    return Expr(mant + (m.group(3) or ""), "real")


# ---------------------------------------------------------------------------
# subroutines
class Var:
    def __init__(self, name, typ, dims=None, arg=False):
        self.name, self.typ, self.dims, self.arg = name, typ, dims, arg
        self.ptr = False  # a scalar POINTER local: held as a C pointer, read through it


class Sub:
    INTRINSIC_REAL = {"sqrt": "sqrt", "tanh": "tanh", "exp": "exp", "log": "log"}

    def __init__(self, name, args):
        self.name, self.args = name, args
        self.vars = {}
        self.body = []
        self.loopvars = set()

    # references -----------------------------------------------------------
    def ref(self, name, args):
        if name in self.vars:
            v = self.vars[name]
            if args is None:
                if v.dims:
                    return Expr("ARRAY:" + name, "array")
                code = ("(*%s)" % name) if ((v.arg or v.ptr) and v.typ != "char") else name
                return Expr(code, v.typ if v.typ != "char" else "str")
            if not v.dims:
                if v.typ == "char":
                    return Expr(name, "str")
                raise TranslateError("scalar %s indexed" % name)
            if any(isinstance(a, tuple) for a in args):
                return Expr(("SECTION", name, args), "section")
            return Expr(self.index(v, [a.code for a in args]), v.typ)
        if args is None:
            raise TranslateError("unknown name %s in %s" % (name, self.name))
        return self.intrinsic(name, args)

    def index(self, v, idx):
        if len(idx) != len(v.dims):
            raise TranslateError("rank mismatch for %s" % v.name)
        terms = []
        for k, code in enumerate(idx):
            off = "((%s) - %s_lo%d)" % (code, v.name, k)
            stride = "*".join("%s_n%d" % (v.name, q) for q in range(k))
            terms.append(off if not stride else "%s*%s" % (off, stride))
        return "%s[%s]" % (v.name, " + ".join(terms))

    def intrinsic(self, name, args):
        a = args
        if name in self.INTRINSIC_REAL:
            return Expr("%s((double)%s)" % (self.INTRINSIC_REAL[name], a[0].code), "real")
        if name == "abs":
            return Expr(("abs(%s)" if a[0].typ == "int" else "fabs(%s)") % a[0].code, a[0].typ)
        if name in ("max", "min"):
            typ = "int" if all(x.typ == "int" for x in a) else "real"
            f = ("f_imax" if name == "max" else "f_imin") if typ == "int" else ("f_max" if name == "max" else "f_min")
            code = a[0].code
            for x in a[1:]:
                code = "%s(%s, %s)" % (f, code, x.code)
            return Expr(code, typ)
        if name == "sign":
            if a[0].typ == "int" and a[1].typ == "int":
                return Expr("f_isign(%s, %s)" % (a[0].code, a[1].code), "int")
            return Expr("f_sign(%s, %s)" % (a[0].code, a[1].code), "real")
        if name in ("float", "real", "dble"):
            return Expr("((double)(%s))" % a[0].code, "real")
        if name in ("int", "nint"):
            f = "(int)" if name == "int" else "(int)lround"
            return Expr("(%s(%s))" % (f, a[0].code), "int")
        if name == "mod":
            if a[0].typ == "int":
                return Expr("((%s) %% (%s))" % (a[0].code, a[1].code), "int")
            return Expr("fmod(%s, %s)" % (a[0].code, a[1].code), "real")
        raise TranslateError("unknown function %s in %s" % (name, self.name))

    def expr(self, s):
        p = ExprParser(tokenize(s), self)
        e = p.parse()
        if p.i != len(p.t):
            raise TranslateError("trailing tokens in %r" % s)
        return e


def _split_top(s, sep=","):
    parts, depth, cur, q = [], 0, [], None
    for ch in s:
        if q:
            cur.append(ch)
            if ch == q:
                q = None
            continue
        if ch in "'\"":
            q = ch
        elif ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        if ch == sep and depth == 0:
            parts.append("".join(cur).strip())
            cur = []
        else:
            cur.append(ch)
    if "".join(cur).strip():
        parts.append("".join(cur).strip())
    return parts


DECL = re.compile(r"^(integer|real\s*\*\s*8|real\s*\(\s*8\s*\)|real|character\s*\(\s*len\s*=\s*\d+\s*\)|character"
                  r"|logical|double\s+precision)\b(.*)$", re.I)


def parse_dims(spec):
    dims = []
    for d in _split_top(spec):
        if ":" in d:
            lo, hi = d.split(":", 1)
        else:
            lo, hi = "1", d
        dims.append((lo.strip(), hi.strip()))
    return dims


class Translator:
    def __init__(self):
        self.subs = []

    def translate_text(self, text, only=None):
        stmts = logical_lines(text)
        i = 0
        while i < len(stmts):
            m = re.match(r"^subroutine\s+(\w+)\s*\((.*)\)\s*$", stmts[i], re.I)
            if not m:
                i += 1
                continue
            name = m.group(1).lower()
            args = [a.strip().lower() for a in m.group(2).split(",") if a.strip()]
            j = i + 1
            while not re.match(r"^end\s*subroutine", stmts[j], re.I):
                j += 1
            if only is None or name in only:
                self.subs.append(self._subroutine(name, args, stmts[i + 1:j]))
            i = j + 1

    # -----------------------------------------------------------------------
    def _subroutine(self, name, args, stmts):
        sub = Sub(name, args)
        body = []
        for s in stmts:
            low = s.lower()
            if re.match(r"^(implicit\s+none|intrinsic\b|external\b)", low):
                continue
            m = DECL.match(s)
            if m and "::" in s:
                attrs = s.split("::", 1)[0][len(m.group(1)):]
                names = s.split("::", 1)[1]
                self._decl(sub, m.group(1), attrs, names)
                if re.search(r"\bpointer\b", attrs, re.I):
                    for n in _split_top(names):
                        v = sub.vars[n.strip().lower()]
                        if v.dims:
                            raise TranslateError("array pointer %s not supported" % v.name)
                        v.ptr = True
                continue
            body.append(s)
        for a in args:
            if a not in sub.vars:
                raise TranslateError("argument %s of %s undeclared" % (a, name))
            sub.vars[a].arg = True
        sub.body = body
        return sub

    def _decl(self, sub, typ, attrs, names):
        t = typ.lower().replace(" ", "")
        if t.startswith("integer"):
            ty = "int"
        elif t.startswith("character"):
            ty = "char"
        elif t.startswith("logical"):
            ty = "int"
        else:
            ty = "real"
        dims = None
        for at in _split_top(attrs.strip().lstrip(",")):
            m = re.match(r"^dimension\s*\((.*)\)$", at.strip(), re.I)
            if m:
                dims = parse_dims(m.group(1))
        for nm in _split_top(names):
            nm = nm.strip()
            m = re.match(r"^(\w+)\s*\((.*)\)$", nm)
            if m:
                sub.vars[m.group(1).lower()] = Var(m.group(1).lower(), ty, parse_dims(m.group(2)))
            else:
                nm = nm.split("=")[0].strip().lower()
                sub.vars[nm] = Var(nm, ty, dims)

    # -----------------------------------------------------------------------
    def emit(self):
        out = [PRELUDE]
        for sub in self.subs:
            out.append(self._emit_sub(sub))
        return "\n".join(out)

    def _ctype(self, v):
        return {"real": "double", "int": "int", "char": "char"}[v.typ]

    def _emit_sub(self, sub):
        params = []
        for a in sub.args:
            v = sub.vars[a]
            if v.typ == "char":
                params.append("const char* %s" % a)
            else:
                params.append("%s* %s" % (self._ctype(v), a))
        lines = ["void ref_%s(%s) {" % (sub.name, ", ".join(params))]
        # scalar locals first (array extents may use them? only args)
        for v in sub.vars.values():
            if v.arg or v.dims:
                continue
            if v.ptr:
                lines.append("  %s* %s = 0;" % (self._ctype(v), v.name))
                continue
            if v.typ == "char":
                lines.append("  char %s[64] = {0};" % v.name)
            else:
                lines.append("  %s %s = 0;" % (self._ctype(v), v.name))
        # array extents (only depend on integer arguments)
        allocs = []
        for v in sub.vars.values():
            if not v.dims:
                continue
            for k, (lo, hi) in enumerate(v.dims):
                lines.append("  const int %s_lo%d = %s;" % (v.name, k, sub.expr(lo).code))
                lines.append("  const int %s_n%d = (%s) - %s_lo%d + 1;" % (v.name, k, sub.expr(hi).code, v.name, k))
            size = "*".join("(size_t)%s_n%d" % (v.name, k) for k in range(len(v.dims)))
            if not v.arg:
                lines.append("  %s* %s = (%s*)calloc(%s, sizeof(%s));" % (self._ctype(v), v.name, self._ctype(v), size,
                                                                          self._ctype(v)))
                allocs.append(v.name)
            lines.append("  const size_t %s_size = %s; (void)%s_size;" % (v.name, size, v.name))
        self._block(sub, sub.body, lines, 1)
        for a in allocs:
            lines.append("  free(%s);" % a)
        lines.append("}")
        return "\n".join(lines)

    def _block(self, sub, stmts, lines, ind):
        # named DO constructs ("name: do ...", "enddo name"): drop the label
        stmts = [re.sub(r"^\w+\s*:\s*(?=do\b)", "", x, flags=re.I) for x in stmts]
        i = 0
        pad = "  " * ind
        while i < len(stmts):
            s = stmts[i]
            low = s.lower()
            m = re.match(r"^do\s+(\w+)\s*=\s*(.*)$", s, re.I)
            if m and not re.match(r"^do\s+while", low):
                depth, j = 1, i + 1
                while j < len(stmts):
                    l2 = stmts[j].lower()
                    if re.match(r"^do\s+\w+\s*=", l2):
                        depth += 1
                    elif re.match(r"^(end\s*do|enddo)\b", l2):
                        depth -= 1
                        if depth == 0:
                            break
                    j += 1
                var = m.group(1).lower()
                rng = _split_top(m.group(2))
                a, b = sub.expr(rng[0]).code, sub.expr(rng[1]).code
                st = sub.expr(rng[2]).code if len(rng) > 2 else "1"
                v = sub.ref(var, None).code
                lines.append("%s{ const int _e%d = %s, _s%d = %s;" % (pad, ind, b, ind, st))
                lines.append("%s  for (%s = %s; _s%d > 0 ? %s <= _e%d : %s >= _e%d; %s += _s%d) {" %
                             (pad, v, a, ind, v, ind, v, ind, v, ind))
                self._block(sub, stmts[i + 1:j], lines, ind + 2)
                lines.append("%s  }" % pad)
                lines.append("%s}" % pad)
                i = j + 1
                continue
            m = re.match(r"^if\s*\((.*)\)\s*then$", s, re.I)
            if m:
                # collect branches
                depth, j = 1, i + 1
                branches, start, cond = [], i + 1, m.group(1)
                while j < len(stmts):
                    l2 = stmts[j].lower()
                    if re.match(r"^if\s*\(.*\)\s*then$", l2):
                        depth += 1
                    elif re.match(r"^(end\s*if|endif)\b", l2):
                        depth -= 1
                        if depth == 0:
                            branches.append((cond, stmts[start:j]))
                            break
                    elif depth == 1 and re.match(r"^else\s*if\s*\(.*\)\s*then$", l2):
                        branches.append((cond, stmts[start:j]))
                        cond = re.match(r"^else\s*if\s*\((.*)\)\s*then$", stmts[j], re.I).group(1)
                        start = j + 1
                    elif depth == 1 and re.match(r"^else$", l2):
                        branches.append((cond, stmts[start:j]))
                        cond = None
                        start = j + 1
                    j += 1
                for k, (c, body) in enumerate(branches):
                    if k == 0:
                        lines.append("%sif (%s) {" % (pad, sub.expr(c).code))
                    elif c is not None:
                        lines.append("%s} else if (%s) {" % (pad, sub.expr(c).code))
                    else:
                        lines.append("%s} else {" % pad)
                    self._block(sub, body, lines, ind + 1)
                lines.append("%s}" % pad)
                i = j + 1
                continue
            m = re.match(r"^if\s*\((.*)$", s, re.I)
            if m:
                # one-line IF (cond) stmt
                rest = s[s.index("(") :]
                depth, k = 0, 0
                for k, ch in enumerate(rest):
                    if ch == "(":
                        depth += 1
                    elif ch == ")":
                        depth -= 1
                        if depth == 0:
                            break
                cond, stmt = rest[1:k], rest[k + 1:].strip()
                lines.append("%sif (%s) {" % (pad, sub.expr(cond).code))
                self._block(sub, [stmt], lines, ind + 1)
                lines.append("%s}" % pad)
                i += 1
                continue
            m = re.match(r"^call\s+(\w+)\s*\((.*)\)$", s, re.I)
            if m:
                lines.append(pad + self._call(sub, m.group(1).lower(), m.group(2)))
                i += 1
                continue
            if re.match(r"^(return|continue)$", low):
                if low == "return":
                    raise TranslateError("RETURN not supported")
                i += 1
                continue
            if "=>" in s:
                m = re.match(r"^(\w+)\s*=>\s*(\w+)$", s)
                p, q = (sub.vars.get(m.group(1).lower()), sub.vars.get(m.group(2).lower())) if m else (None, None)
                if p is None or q is None or not p.ptr or q.dims or q.typ != p.typ:
                    raise TranslateError("pointer assignment not supported: %s" % s)
                lines.append("%s%s = %s%s;" % (pad, p.name, "" if (q.arg or q.ptr) else "&", q.name))
                i += 1
                continue
            self._assign(sub, s, lines, pad)
            i += 1

    def _call(self, sub, name, argstr):
        args = _split_top(argstr)
        if name.startswith("push"):
            e = sub.expr(args[0])
            kind = "r" if e.typ == "real" else "i"
            return "f_push_%s((%s));" % (kind, e.code)
        if name.startswith("pop"):
            e = sub.expr(args[0])
            kind = "r" if e.typ == "real" else "i"
            return "%s = f_pop_%s();" % (e.code, kind)
        callee = next((c for c in self.subs if c.name == name), None)
        if callee is None:
            raise TranslateError("unsupported CALL %s" % name)
        if len(args) != len(callee.args):
            raise TranslateError("CALL %s: %d arguments for %d" % (name, len(args), len(callee.args)))
        # Fortran passes by reference: whole arrays by their base pointer,
        # scalar variables by address, expressions through a temporary
        pre, actual = [], []
        for k, a in enumerate(args):
            a = a.strip()
            if re.match(r"^\w+$", a) and a.lower() in sub.vars:
                v = sub.vars[a.lower()]
                if v.dims or v.typ == "char" or v.arg or v.ptr:
                    actual.append(v.name)
                else:
                    actual.append("&" + v.name)
                continue
            e = sub.expr(a)
            ct = "int" if e.typ == "int" else "double"
            pre.append("%s _ca%d = (%s);" % (ct, k, e.code))
            actual.append("&_ca%d" % k)
        return "{ %s ref_%s(%s); }" % (" ".join(pre), name, ", ".join(actual))

    def _assign(self, sub, s, lines, pad):
        lhs, rhs = _split_assign(s)
        le = sub.expr(lhs)
        if le.typ in ("array", "section"):
            name = le.code[6:] if le.typ == "array" else le.code[1]
            v = sub.vars[name]
            if le.typ == "array":
                idx = [("section", None, None)] * len(v.dims)
            else:
                idx = le.code[2]
            loops, sub_idx = [], []
            for k, a in enumerate(idx):
                if isinstance(a, tuple):
                    lo = a[1].code if a[1] is not None else "%s_lo%d" % (name, k)
                    hi = a[2].code if a[2] is not None else "(%s_lo%d + %s_n%d - 1)" % (name, k, name, k)
                    lv = "_q%d" % k
                    loops.append((lv, lo, hi))
                    sub_idx.append((k, lv))
                else:
                    sub_idx.append((k, None))
            lhs_idx = []
            for k, a in enumerate(idx):
                lhs_idx.append(dict(sub_idx)[k] if isinstance(a, tuple) else a.code)
            target = sub.index(v, lhs_idx)
            rcode = self._section_rhs(sub, rhs, [lv for _, lv, _ in [(0, l[0], 0) for l in loops]], loops)
            # evaluate into a temporary buffer first (Fortran semantics)
            lines.append("%s{" % pad)
            for lv, lo, hi in loops:
                lines.append("%s  for (int %s = %s; %s <= %s; ++%s)" % (pad, lv, lo, lv, hi, lv))
            lines.append("%s    %s = %s;" % (pad, target, rcode))
            lines.append("%s}" % pad)
            return
        re_ = sub.expr(rhs)
        if re_.typ == "str":
            raise TranslateError("string assignment")
        lines.append("%s%s = %s;" % (pad, le.code, re_.code))

    def _section_rhs(self, sub, rhs, loopvars, loops):
        """Rewrite sections / whole arrays on the right-hand side to elements,
        matching the k-th section dimension with the k-th LHS loop."""
        toks = tokenize(rhs)
        p = ExprParser(toks, SectionSub(sub, loops))
        e = p.parse()
        return e.code


class SectionSub:
    """Reference resolver that turns array sections into elements indexed by
    the loop variables of the enclosing section assignment."""

    def __init__(self, sub, loops):
        self.sub, self.loops = sub, loops

    def ref(self, name, args):
        v = self.sub.vars.get(name)
        if v is not None and v.dims:
            if args is None:
                args = [("section", None, None)] * len(v.dims)
            if any(isinstance(a, tuple) for a in args):
                idx, n = [], 0
                for k, a in enumerate(args):
                    if isinstance(a, tuple):
                        lv, lo_l, _ = self.loops[n]
                        lo = a[1].code if a[1] is not None else "%s_lo%d" % (name, k)
                        # element = lower bound of this section + offset of the loop
                        idx.append("(%s) + (%s - (%s))" % (lo, lv, lo_l))
                        n += 1
                    else:
                        idx.append(a.code)
                return Expr(self.sub.index(v, idx), v.typ)
        return self.sub.ref(name, args)

    def intrinsic(self, name, args):
        return self.sub.intrinsic(name, args)


def _split_assign(s):
    depth = 0
    for k, ch in enumerate(s):
        if ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        elif ch == "=" and depth == 0:
            nxt = s[k + 1] if k + 1 < len(s) else ""
            prv = s[k - 1] if k > 0 else ""
            if nxt not in "=>" and prv not in "<>/=":
                return s[:k].strip(), s[k + 1:].strip()
    raise TranslateError("not an assignment: %r" % s)


PRELUDE = r"""/* Generated by oracle/ref_translate.py from the reference's Fortran source;
 * test infrastructure only, never committed. */
#include <math.h>
#include <stdlib.h>
#include <string.h>
static inline double f_max(double a, double b) { return a > b ? a : (b > a ? b : a); }
static inline double f_min(double a, double b) { return a < b ? a : (b < a ? b : a); }
static inline int f_imax(int a, int b) { return a > b ? a : b; }
static inline int f_imin(int a, int b) { return a < b ? a : b; }
static inline double f_sign(double a, double b) { return (b >= 0.0) ? fabs(a) : -fabs(a); }
static inline int f_isign(int a, int b) { return (b >= 0) ? abs(a) : -abs(a); }
static inline double f_sq(double a) { return a * a; }
static inline double f_powi(double a, int n) { double r = 1.0; for (int k = 0; k < n; ++k) r *= a; return r; }
static inline int f_ipowi(int a, int n) { int r = 1; for (int k = 0; k < n; ++k) r *= a; return r; }
static double* f_stk_r = 0; static long f_nr = 0, f_cr = 0;
static int* f_stk_i = 0; static long f_ni = 0, f_ci = 0;
static void f_push_r(double x) { if (f_nr == f_cr) { f_cr = f_cr ? 2 * f_cr : 1024; f_stk_r = (double*)realloc(f_stk_r, f_cr * sizeof(double)); } f_stk_r[f_nr++] = x; }
static double f_pop_r(void) { return f_stk_r[--f_nr]; }
static void f_push_i(int x) { if (f_ni == f_ci) { f_ci = f_ci ? 2 * f_ci : 1024; f_stk_i = (int*)realloc(f_stk_i, f_ci * sizeof(int)); } f_stk_i[f_ni++] = x; }
static int f_pop_i(void) { return f_stk_i[--f_ni]; }
"""
