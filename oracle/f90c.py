"""f90c: translate the Fortran 90 subset of RAM's kinetic-step routines to C.

TEST INFRASTRUCTURE ONLY (part of the oracle): no product code imports it.

RAM-SCB is Fortran and no Fortran compiler exists on the machines this
project is built and tested on.  This translator reads the reference's own
source files where they lie and writes one C file (plus a gcc build of it)
into ``oracle/_ref/``, so that the reference's routines themselves -- not a
restatement -- can run on the CPU, pin the oracle and the CUDA path, and
serve as the timed reference arm.  Nothing it reads is copied into the
repository: its output directory is git-ignored.

Semantics follow gfortran as the reference builds it (``src/Makefile:27``:
``-fdefault-real-8 -fdefault-double-8 -finit-local-zero``):

* every REAL (any kind, every literal) is an IEEE double; integers are
  32-bit; locals start at zero; module variables live in zeroed storage;
* expressions keep the Fortran parse order (left to right, parentheses
  respected, no contraction: the C is built with ``-ffp-contract=off``);
* ``x**n`` with a constant integer n expands into the multiplication chain
  of gfortran's constant-power expansion (x*x, x*(x*x), (x*x)*(x*x), ...),
  ``x**y`` with a real y calls ``pow``; intrinsics call the same libm;
* ``!$OMP PARALLEL DO`` becomes ``#pragma omp parallel for`` and
  ``!$OMP THREADPRIVATE`` variables become thread-local.

Only the procedures named on the command line (and the driver module of
``oracle/refdriver.f90``) are translated; a call to any other procedure
becomes a stub that counts its calls and does nothing, and a statement the
subset does not cover becomes a runtime failure, so an untaken branch may
hold anything while a taken one fails loudly.  I/O statements are no-ops.
"""
from __future__ import annotations

import argparse
import os
import re
import subprocess
import sys
from dataclasses import dataclass, field
from pathlib import Path


class Unsupported(Exception):
    pass


# ---------------------------------------------------------------- reading
@dataclass
class Stmt:
    file: str
    line: int
    text: str                 # comments removed, continuations joined
    omp: str = ""             # lower-case directive text for !$omp lines

    @property
    def where(self):
        return f"{os.path.basename(self.file)}:{self.line}"


def _strip_comment(line: str) -> str:
    q = None
    for i, ch in enumerate(line):
        if q:
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
        elif ch == "!":
            return line[:i]
    return line


def _split_top(s: str, sep: str):
    """Split at sep outside quotes and parentheses."""
    out, depth, q, cur = [], 0, None, []
    for ch in s:
        if q:
            cur.append(ch)
            if ch == q:
                q = None
            continue
        if ch in "'\"":
            q = ch
        elif ch in "([":
            depth += 1
        elif ch in ")]":
            depth -= 1
        elif ch == sep and depth == 0:
            out.append("".join(cur))
            cur = []
            continue
        cur.append(ch)
    out.append("".join(cur))
    return out


def read_statements(path: str):
    raw = Path(path).read_text(encoding="latin-1").split("\n")
    out, buf, start = [], "", 0
    for i, line in enumerate(raw, 1):
        line = line.replace("\t", " ")
        s = line.strip()
        if s.lower().startswith("!$omp"):
            if not buf:
                out.append(Stmt(path, i, "", omp=s[5:].strip().lower()))
            continue
        code = _strip_comment(line).rstrip()
        if not code.strip():
            continue
        if buf:
            c = code.lstrip()
            if c.startswith("&"):
                c = c[1:]
        else:
            c = code
            start = i
        if c.endswith("&"):
            buf += c[:-1]
            continue
        buf += c
        for part in _split_top(buf, ";"):
            t = part.strip()
            m = re.match(r"^(\d+)\s+(.*)$", t)
            if m:  # statement label
                t = m.group(2)
            if t:
                out.append(Stmt(path, start, t))
        buf = ""
    return out


# ---------------------------------------------------------------- lexing
_TOK = re.compile(r"""
  (?P<ws>\s+)
 |(?P<str>'(?:[^']|'')*'|"(?:[^"]|"")*")
 |(?P<dot>\.(?:and|or|not|eqv|neqv|eq|ne|lt|le|gt|ge|true|false)\.(?:_\w+)?)
 |(?P<num>(?:\d+\.?\d*|\.\d+)(?:[eEdD][+-]?\d+)?(?:_\w+)?)
 |(?P<name>[A-Za-z_]\w*)
 |(?P<op>\*\*|//|==|/=|<=|>=|=>|::|\(/|/\)|[-+*/()<>=,:%\[\]])
""", re.X | re.I)


@dataclass
class Tok:
    kind: str
    val: str


def tokenize(s: str):
    toks, i = [], 0
    while i < len(s):
        m = _TOK.match(s, i)
        if not m:
            raise Unsupported(f"cannot tokenize at {s[i:i + 20]!r}")
        kind = m.lastgroup
        v = m.group(kind)
        if kind == "num":
            # '1.eq.2': the '.' belongs to the operator
            mm = re.match(r"(\d+)\.(and|or|not|eqv|neqv|eq|ne|lt|le|gt|ge|true|false)\.", s[i:], re.I)
            if mm:
                v = mm.group(1)
                m = None
                toks.append(Tok("num", v))
                i += len(v)
                continue
        i = m.end()
        if kind == "ws":
            continue
        if kind == "op" and v == "(/":
            toks += [Tok("op", "("), Tok("op", "/")]
            continue
        if kind == "op" and v == "/)":
            # '/)' closes an array constructor; a division followed by ')'
            # cannot occur in valid code
            toks += [Tok("op", "/"), Tok("op", ")")]
            continue
        toks.append(Tok(kind, v.lower() if kind in ("dot", "name") else v))
    return toks


# ---------------------------------------------------------------- expressions
@dataclass
class Num:
    text: str
    is_real: bool


@dataclass
class Str:
    s: str


@dataclass
class Bool:
    v: bool


@dataclass
class Ref:          # name [(args)] {% name [(args)]}
    parts: list     # [(name, args or None)]


@dataclass
class Bin:
    op: str
    l: object
    r: object


@dataclass
class Un:
    op: str
    e: object


@dataclass
class Rng:          # section lo:hi[:step]; None = open
    lo: object
    hi: object
    st: object = None


@dataclass
class Kw:
    name: str
    e: object


@dataclass
class Cons:
    items: list


class Parser:
    def __init__(self, toks):
        self.t = toks
        self.i = 0

    def peek(self, k=0):
        j = self.i + k
        return self.t[j] if j < len(self.t) else Tok("eof", "")

    def eat(self, val=None):
        tk = self.peek()
        if val is not None and tk.val != val:
            raise Unsupported(f"expected {val!r}, got {tk.val!r}")
        self.i += 1
        return tk

    def at(self, val):
        return self.peek().val == val

    def done(self):
        return self.i >= len(self.t)

    # precedence: eqv < or < and < not < rel < concat < add < mul < pow < unary
    def expr(self):
        e = self.e_or()
        while self.peek().val in (".eqv.", ".neqv."):
            op = self.eat().val
            e = Bin(op, e, self.e_or())
        return e

    def e_or(self):
        e = self.e_and()
        while self.at(".or."):
            self.eat()
            e = Bin(".or.", e, self.e_and())
        return e

    def e_and(self):
        e = self.e_not()
        while self.at(".and."):
            self.eat()
            e = Bin(".and.", e, self.e_not())
        return e

    def e_not(self):
        if self.at(".not."):
            self.eat()
            return Un(".not.", self.e_not())
        return self.e_rel()

    _REL = {"==": "==", ".eq.": "==", "/=": "!=", ".ne.": "!=", "<": "<", ".lt.": "<",
            "<=": "<=", ".le.": "<=", ">": ">", ".gt.": ">", ">=": ">=", ".ge.": ">="}

    def e_rel(self):
        e = self.e_cat()
        if self.peek().val in self._REL:
            op = self._REL[self.eat().val]
            e = Bin(op, e, self.e_cat())
        return e

    def e_cat(self):
        e = self.e_add()
        while self.at("//"):
            self.eat()
            e = Bin("//", e, self.e_add())
        return e

    def e_add(self):
        if self.peek().val in ("+", "-"):
            op = self.eat().val
            e = self.e_mul()
            e = Un(op, e)
        else:
            e = self.e_mul()
        while self.peek().val in ("+", "-"):
            op = self.eat().val
            e = Bin(op, e, self.e_mul())
        return e

    def e_mul(self):
        e = self.e_pow()
        while self.peek().val in ("*", "/") and not (self.peek().val == "/" and self.peek(1).val == ")"):
            op = self.eat().val
            e = Bin(op, e, self.e_pow())
        return e

    def e_pow(self):
        b = self.primary()
        if self.at("**"):
            self.eat()
            # right associative; a unary sign may follow '**'
            if self.peek().val in ("+", "-"):
                op = self.eat().val
                return Bin("**", b, Un(op, self.e_pow()))
            return Bin("**", b, self.e_pow())
        return b

    def primary(self):
        tk = self.peek()
        if tk.kind == "num":
            self.eat()
            txt = tk.val
            is_real = bool(re.search(r"[.eEdD]", txt.split("_")[0]))
            return Num(txt, is_real)
        if tk.kind == "str":
            self.eat()
            q = tk.val[0]
            return Str(tk.val[1:-1].replace(q + q, q))
        if tk.kind == "dot" and tk.val.split("_")[0] in (".true.", ".false."):
            self.eat()
            return Bool(tk.val.startswith(".true."))
        if tk.val == "(":
            if self.peek(1).val == "/":
                self.eat()
                self.eat()
                items = []
                while not (self.at("/") and self.peek(1).val == ")"):
                    items.append(self.expr())
                    if self.at(","):
                        self.eat()
                self.eat("/")
                self.eat(")")
                return Cons(items)
            self.eat()
            e = self.expr()
            self.eat(")")
            return Un("()", e)
        if tk.val == "[":
            self.eat()
            items = []
            while not self.at("]"):
                items.append(self.expr())
                if self.at(","):
                    self.eat()
            self.eat("]")
            return Cons(items)
        if tk.kind == "name":
            parts = []
            while True:
                name = self.eat().val
                args = None
                if self.at("("):
                    args = self.arglist()
                parts.append((name, args))
                if self.at("%"):
                    self.eat()
                    if self.peek().kind != "name":
                        raise Unsupported("bad component reference")
                    continue
                break
            return Ref(parts)
        raise Unsupported(f"unexpected token {tk.val!r}")

    def arglist(self):
        self.eat("(")
        args = []
        if self.at(")"):
            self.eat()
            return args
        while True:
            args.append(self.arg())
            if self.at(","):
                self.eat()
                continue
            self.eat(")")
            return args

    def arg(self):
        if self.peek().kind == "name" and self.peek(1).val == "=" and self.peek(2).val != "=":
            name = self.eat().val
            self.eat("=")
            return Kw(name, self.expr())
        lo = None
        if not self.at(":"):
            lo = self.expr()
            if not self.at(":"):
                return lo
        self.eat(":")
        hi = None
        if not (self.at(",") or self.at(")") or self.at(":")):
            hi = self.expr()
        st = None
        if self.at(":"):
            self.eat()
            st = self.expr()
        return Rng(lo, hi, st)


def parse_expr(text):
    p = Parser(tokenize(text))
    e = p.expr()
    if not p.done():
        raise Unsupported(f"trailing tokens in {text!r}")
    return e


# ---------------------------------------------------------------- symbols
@dataclass
class Sym:
    name: str
    base: str                 # 'i' 'r' 'l' 'c' or 't:<type>'
    clen: object = None       # character length (int) or None
    dims: list = None         # None scalar; list of (lo, hi) ASTs, hi None = deferred
    alloc: bool = False
    param: bool = False
    init: object = None
    save: bool = False
    module: str = None
    dummy: bool = False
    intent: str = ""
    value: object = None      # constant value of a parameter
    data: list = None
    tls: bool = False
    cname: str = ""

    @property
    def rank(self):
        return 0 if self.dims is None else len(self.dims)


@dataclass
class TypeDef:
    name: str
    fields: dict              # name -> Sym


@dataclass
class Proc:
    name: str
    module: str
    args: list
    is_func: bool
    result: str
    body: list                # statements after the specification part
    spec: list
    syms: dict = field(default_factory=dict)
    uses: list = field(default_factory=list)


@dataclass
class Module:
    name: str
    file: str
    spec: list
    procs: dict
    syms: dict = field(default_factory=dict)
    types: dict = field(default_factory=dict)
    uses: list = field(default_factory=list)
    threadprivate: set = field(default_factory=set)


_DECL = re.compile(r"^(integer|real|logical|character|double\s*precision|type\s*\(|complex)\b", re.I)
_SKIP_SPEC = re.compile(r"^(implicit|public|private|intrinsic|external|save\s*$|sequence|contains|include)\b", re.I)
_IO = re.compile(r"^(write|print|read|open|close|format|flush|inquire|rewind|backspace|endfile)\b", re.I)


def parse_modules(path):
    """Split a file into modules; each module into its specification part
    and its procedures (statement lists)."""
    stmts = read_statements(path)
    mods = {}
    i = 0
    while i < len(stmts):
        st = stmts[i]
        low = st.text.lower()
        m = re.match(r"^module\s+(\w+)\s*$", low)
        if not m:
            i += 1
            continue
        name = m.group(1)
        i += 1
        spec, procs = [], {}
        while i < len(stmts) and not re.match(r"^contains\s*$", stmts[i].text.lower()) and \
                not re.match(r"^end\s*module\b", stmts[i].text.lower()):
            spec.append(stmts[i])
            i += 1
        if i < len(stmts) and stmts[i].text.lower().startswith("contains"):
            i += 1
            while i < len(stmts) and not re.match(r"^end\s*module\b", stmts[i].text.lower()):
                i, pr = _parse_proc(stmts, i, name)
                if pr is not None:
                    procs[pr.name] = pr
        i += 1
        mods[name] = Module(name, path, spec, procs)
    return mods


_PROC_HDR = re.compile(
    r"^(?:(?:recursive|pure|elemental)\s+)*(?:(?:integer|real|logical|double\s*precision)\s*(?:\([^)]*\))?\s+)?"
    r"(subroutine|function)\s+(\w+)\s*(?:\(([^)]*)\))?\s*(?:result\s*\(\s*(\w+)\s*\))?\s*$", re.I)


def _parse_proc(stmts, i, modname):
    st = stmts[i]
    m = _PROC_HDR.match(st.text.strip())
    if not m:
        return i + 1, None
    kind, name = m.group(1).lower(), m.group(2).lower()
    args = [a.strip().lower() for a in (m.group(3) or "").split(",") if a.strip()]
    result = (m.group(4) or name).lower()
    i += 1
    spec, body = [], []
    depth = 0
    in_spec = True
    bad = False
    while i < len(stmts):
        t = stmts[i].text.lower().strip()
        if re.match(r"^end\s*(subroutine|function)\b", t) or t == "end":
            break
        if re.match(r"^contains\s*$", t):
            # internal procedures: not in the subset; skip them and mark
            # the host procedure untranslatable
            bad = True
            i += 1
            depth = 0
            while i < len(stmts):
                t = stmts[i].text.lower().strip()
                if _PROC_HDR.match(stmts[i].text.strip()):
                    depth += 1
                elif re.match(r"^end\s*(subroutine|function)\b", t) or t == "end":
                    if depth == 0:
                        break
                    depth -= 1
                i += 1
            break
        if in_spec and not stmts[i].omp and (
                t.startswith("use ") or _DECL.match(t) and not re.match(r"^type\s*\(\s*\w+\s*\)\s*=", t)
                or _SKIP_SPEC.match(t) or t.startswith("data ") or t.startswith("data/") or re.match(r"^save\b", t)
                or t.startswith("parameter") or t.startswith("dimension")):
            spec.append(stmts[i])
        else:
            in_spec = False
            body.append(stmts[i])
        i += 1
    pr = Proc(name, modname, args, kind == "function", result, body, spec)
    pr.bad = bad
    return i + 1, pr


# ---------------------------------------------------------------- declarations
def _parse_typespec(s):
    """-> (base, kind/len info, rest) ; s lower-case."""
    m = re.match(r"^(integer|real|logical|complex)\s*(\*\s*\d+|\([^()]*(?:\([^()]*\)[^()]*)*\))?", s)
    if m:
        b = {"integer": "i", "real": "r", "logical": "l", "complex": "x"}[m.group(1)]
        return b, None, s[m.end():]
    m = re.match(r"^double\s*precision", s)
    if m:
        return "r", None, s[m.end():]
    m = re.match(r"^character\s*(\*\s*(\d+)|\(([^()]*)\))?", s)
    if m:
        ln = None
        if m.group(2):
            ln = m.group(2)
        elif m.group(3):
            sp = m.group(3).strip()
            mm = re.match(r"^(?:len\s*=\s*)?([^,]+)", sp)
            ln = mm.group(1).strip() if mm else "1"
        else:
            ln = "1"
        return "c", ln, s[m.end():]
    m = re.match(r"^type\s*\(\s*(\w+)\s*\)", s)
    if m:
        return "t:" + m.group(1), None, s[m.end():]
    raise Unsupported(f"type spec {s[:30]!r}")


def _parse_dims(text):
    dims = []
    for d in _split_top(text, ","):
        d = d.strip()
        if d in (":", "*"):
            dims.append((None, None))
            continue
        parts = _split_top(d, ":")
        if len(parts) == 1:
            dims.append((Num("1", False), parse_expr(parts[0])))
        else:
            lo = parse_expr(parts[0]) if parts[0].strip() else None
            hi = parse_expr(parts[1]) if parts[1].strip() else None
            dims.append((lo, hi))
    return dims


def parse_decl(text):
    """One declaration statement -> list of Sym (module/local unset)."""
    s = text.strip()
    low = s.lower()
    base, ln, rest = _parse_typespec(low)
    rest_orig = s[len(s) - len(rest):]
    attrs, ents = "", rest_orig
    if "::" in rest_orig:
        attrs, ents = rest_orig.split("::", 1)
    attrl = [a.strip().lower() for a in _split_top(attrs, ",") if a.strip()]
    dims_attr, alloc, param, save, intent = None, False, False, False, ""
    for a in attrl:
        if a.startswith("dimension"):
            dims_attr = _parse_dims(a[a.index("(") + 1:a.rindex(")")])
        elif a in ("allocatable", "pointer", "target"):
            alloc = alloc or a != "target"
        elif a == "parameter":
            param = True
        elif a == "save":
            save = True
        elif a.startswith("intent"):
            intent = a[a.index("(") + 1:a.rindex(")")].strip()
    out = []
    for ent in _split_top(ents, ","):
        ent = ent.strip()
        if not ent:
            continue
        init = None
        eq = _split_top(ent, "=")
        if len(eq) > 1 and not ent.lstrip().startswith("=>"):
            # 'x = expr' (not '==')
            idx = _find_assign(ent)
            if idx >= 0:
                init = parse_expr(ent[idx + 1:])
                ent = ent[:idx].strip()
        m = re.match(r"^(\w+)\s*(\((.*)\))?\s*(\*\s*(\d+))?$", ent)
        if not m:
            raise Unsupported(f"entity {ent!r}")
        name = m.group(1).lower()
        dims = _parse_dims(m.group(3)) if m.group(2) else dims_attr
        eln = m.group(5) or ln
        out.append(Sym(name, base, clen=eln, dims=dims, alloc=alloc, param=param, init=init,
                       save=save or (init is not None and not param), intent=intent))
    return out


def _find_assign(s):
    """Index of the assignment '=' at top level, or -1."""
    depth, q = 0, None
    for i, ch in enumerate(s):
        if q:
            if ch == q:
                q = None
            continue
        if ch in "'\"":
            q = ch
        elif ch in "([":
            depth += 1
        elif ch in ")]":
            depth -= 1
        elif ch == "=" and depth == 0:
            prev = s[i - 1] if i else ""
            nxt = s[i + 1] if i + 1 < len(s) else ""
            if prev in "=/<>" or nxt in "=>":
                continue
            return i
    return -1


# ---------------------------------------------------------------- C helpers
PRELUDE = r"""/* Generated by oracle/f90c.py from the reference's Fortran sources.
 * Test infrastructure: do not edit, do not commit. */
#include <math.h>
#include <float.h>
#include <limits.h>
#include <setjmp.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct { void* p; int esz, rank; long lb[7], ub[7], sm[7]; } RefArr;
typedef struct { const char* p; int n; } RefStr;

static char ref_errbuf[512];
static int ref_errset;
static jmp_buf ref_jb;
static __thread int ref_in_parallel;

static void ref_fail(const char* where) {
  if (!ref_errset) { snprintf(ref_errbuf, sizeof ref_errbuf, "%s", where); ref_errset = 1; }
  if (!ref_in_parallel) longjmp(ref_jb, 1);
}
#ifdef REF_CHECK
static long ref_chk(const RefArr* a, int d, long i, const char* where) {
  if (!a->p || i < a->lb[d] || i > a->ub[d]) {
    char b[400];
    snprintf(b, sizeof b, "%s: index %ld of dim %d outside [%ld,%ld]%s", where, i, d + 1, a->lb[d], a->ub[d],
             a->p ? "" : " (not allocated)");
    ref_fail(b);
  }
  return i;
}
#define RC(a, d, i, w) ref_chk(&(a), d, (i), w)
#else
#define RC(a, d, i, w) (i)
#endif
static inline long ref_o1(const RefArr* a, long i) { return i - a->lb[0]; }
static inline long ref_o2(const RefArr* a, long i, long j) { return (i - a->lb[0]) + a->sm[1] * (j - a->lb[1]); }
static inline long ref_o3(const RefArr* a, long i, long j, long k) {
  return (i - a->lb[0]) + a->sm[1] * (j - a->lb[1]) + a->sm[2] * (k - a->lb[2]);
}
static inline long ref_o4(const RefArr* a, long i, long j, long k, long l) {
  return (i - a->lb[0]) + a->sm[1] * (j - a->lb[1]) + a->sm[2] * (k - a->lb[2]) + a->sm[3] * (l - a->lb[3]);
}
static inline long ref_o5(const RefArr* a, long i, long j, long k, long l, long m) {
  return (i - a->lb[0]) + a->sm[1] * (j - a->lb[1]) + a->sm[2] * (k - a->lb[2]) + a->sm[3] * (l - a->lb[3]) +
         a->sm[4] * (m - a->lb[4]);
}
static void ref_alloc(RefArr* a, int esz, int rank, const long* lb, const long* ub, const char* where) {
  if (a->p) ref_fail(where);  /* ALLOCATE of an allocated array is an error in Fortran */
  long n = 1;
  a->esz = esz; a->rank = rank;
  for (int d = 0; d < rank; ++d) {
    a->lb[d] = lb[d]; a->ub[d] = ub[d];
    a->sm[d] = n;
    long e = ub[d] - lb[d] + 1;
    n *= e > 0 ? e : 0;
  }
  a->p = calloc(n > 0 ? (size_t)n : 1, (size_t)esz);
}
static void ref_dealloc(RefArr* a) { free(a->p); a->p = NULL; }
static long ref_size(const RefArr* a) {
  long n = 1;
  for (int d = 0; d < a->rank; ++d) { long e = a->ub[d] - a->lb[d] + 1; n *= e > 0 ? e : 0; }
  return n;
}
static inline double ref_powi(double x, int m) {  /* binary method, as libgcc's powi */
  unsigned n = m < 0 ? -(unsigned)m : (unsigned)m;
  double y = (n % 2) ? x : 1.0;
  while (n >>= 1) { x = x * x; if (n % 2) y = y * x; }
  return m < 0 ? 1.0 / y : y;
}
static inline int ref_ipow(int b, int e) { int r = 1; if (e < 0) return b == 1 ? 1 : (b == -1 ? (e % 2 ? -1 : 1) : 0); while (e-- > 0) r *= b; return r; }
static inline double ref_maxd(double a, double b) { return b > a ? b : a; }
static inline double ref_mind(double a, double b) { return b < a ? b : a; }
static inline int ref_maxi(int a, int b) { return b > a ? b : a; }
static inline int ref_mini(int a, int b) { return b < a ? b : a; }
static inline double ref_signd(double a, double b) { return copysign(fabs(a), b); }
static inline int ref_signi(int a, int b) { return b >= 0 ? abs(a) : -abs(a); }
static inline int ref_nint(double x) { return (int)lround(x); }
static inline RefStr ref_trim(RefStr s) { while (s.n > 0 && s.p[s.n - 1] == ' ') --s.n; return s; }
static int ref_streq(RefStr a, RefStr b) {
  int n = a.n > b.n ? a.n : b.n;
  for (int i = 0; i < n; ++i) {
    char x = i < a.n ? a.p[i] : ' ', y = i < b.n ? b.p[i] : ' ';
    if (x != y) return 0;
  }
  return 1;
}
static void ref_sassign(char* d, int dn, RefStr s) {
  for (int i = 0; i < dn; ++i) d[i] = i < s.n ? s.p[i] : ' ';
}

#define REF_NSTUB 64
static const char* ref_stub_names[REF_NSTUB];
static long ref_stub_calls[REF_NSTUB];
static int ref_nstub;
static void ref_stub(const char* name) {
#pragma omp critical(ref_stub)
  {
    int i;
    for (i = 0; i < ref_nstub; ++i)
      if (!strcmp(ref_stub_names[i], name)) break;
    if (i == ref_nstub && ref_nstub < REF_NSTUB) ref_stub_names[ref_nstub++] = name;
    if (i < REF_NSTUB) ref_stub_calls[i]++;
  }
}
"""

# Exponent splits of gfortran's constant integer power expansion (the
# optimal addition chains for small n): x**n = x**(n-t) * x**t, t = _POWI[n].
_POWI = {2: 1, 3: 2, 4: 2, 5: 3, 6: 3, 7: 4, 8: 4, 9: 6, 10: 7, 11: 6, 12: 8}

_INTRINSIC = {"abs", "max", "min", "exp", "log", "log10", "sqrt", "sin", "cos", "tan", "asin", "acos", "atan",
              "atan2", "sinh", "cosh", "tanh", "real", "dble", "float", "int", "nint", "floor", "ceiling", "mod",
              "sign", "huge", "tiny", "epsilon", "size", "allocated", "minval", "maxval", "sum", "trim", "merge",
              "kind", "selected_int_kind", "selected_real_kind", "lbound", "ubound", "len", "len_trim", "dmax1",
              "dmin1", "amax1", "amin1", "dabs", "dsqrt", "dexp", "dlog", "dlog10"}


class Ctx:
    """Per-procedure translation state; copies share the temporary counter."""

    def __init__(self, tr, proc, counter=None, loops=None, where=""):
        self.tr = tr
        self.proc = proc
        self.counter = counter if counter is not None else [0]
        self.loops = loops  # elemental loop vars: list of (cvar, lo_code)
        self.where = where

    def newtmp(self, p="_t"):
        self.counter[0] += 1
        return f"{p}{self.counter[0]}"

    def scalar(self):
        return Ctx(self.tr, self.proc, self.counter, None, self.where)

    def with_loops(self, loops):
        return Ctx(self.tr, self.proc, self.counter, loops, self.where)


def _powi_chain(v, n):
    if n == 1:
        return v
    t = _POWI[n]
    return f"({_powi_chain(v, n - t)} * {_powi_chain(v, t)})"


def _powi_py(x, n):
    if n == 0:
        return 1.0
    if n < 0:
        return 1.0 / _powi_py(x, -n)
    if n == 1:
        return x
    if n in _POWI:
        t = _POWI[n]
        return _powi_py(x, n - t) * _powi_py(x, t)
    y = x if n % 2 else 1.0
    while True:
        n >>= 1
        if not n:
            return y
        x = x * x
        if n % 2:
            y = y * x


class Translator:
    def __init__(self, modules: dict, procs: list, stub_ok=()):
        self.mods = modules
        self.want = [p.lower() for p in procs]
        self.types = {}
        self.used_globals = {}    # cname -> Sym
        self.translated = {}      # proc name -> cname

    # ------------------------------------------------------------ scoping
    def setup(self):
        for mn, m in self.mods.items():
            for st in m.spec:
                if st.omp:
                    mm = re.match(r"threadprivate\s*\((.*)\)", st.omp)
                    if mm:
                        m.threadprivate |= {x.strip() for x in mm.group(1).split(",")}
                    continue
            self._spec(m, m.spec, m.syms, m.uses, module=mn, types=m.types)
            self.types.update(m.types)
            for n in m.threadprivate:
                if n in m.syms:
                    m.syms[n].tls = True

    def _spec(self, owner, stmts, syms, uses, module=None, types=None):
        i = 0
        while i < len(stmts):
            st = stmts[i]
            t = st.text.strip()
            low = t.lower()
            i += 1
            if st.omp or not t:
                continue
            try:
                if low.startswith("use ") or low.startswith("use,"):
                    mm = re.match(r"^use\s*(?:,\s*\w+\s*::)?\s*(\w+)\s*(?:,\s*only\s*:\s*(.*))?$", low)
                    if not mm:
                        raise Unsupported("use")
                    only = None
                    if mm.group(2) is not None:
                        only = []
                        for it in mm.group(2).split(","):
                            it = it.strip()
                            if not it:
                                continue
                            if "=>" in it:
                                a, b = [x.strip() for x in it.split("=>")]
                                only.append((a, b))
                            else:
                                only.append((it, it))
                    uses.append((mm.group(1), only))
                    continue
                if re.match(r"^type\s+(?:,\s*\w+\s*)?(?:::)?\s*\w+\s*$", low) and not low.startswith("type("):
                    name = low.split()[-1].replace("::", "").strip()
                    flds = {}
                    while i < len(stmts) and not re.match(r"^end\s*type", stmts[i].text.lower()):
                        for s in parse_decl(stmts[i].text):
                            flds[s.name] = s
                        i += 1
                    i += 1
                    if types is not None:
                        types[name] = TypeDef(name, flds)
                    continue
                if low.startswith("interface"):
                    while i < len(stmts) and not stmts[i].text.lower().startswith("end interface") and \
                            not stmts[i].text.lower().startswith("endinterface"):
                        i += 1
                    i += 1
                    continue
                mm = re.match(r"^save\s*(?:::)?\s*(.*)$", low)
                if mm:
                    names = [x.strip() for x in mm.group(1).split(",") if x.strip()]
                    saves = syms.setdefault("__save__", [])
                    saves.extend(names or ["*"])
                    continue
                if _SKIP_SPEC.match(low):
                    continue
                if low.startswith("data"):
                    self._data(t, syms)
                    continue
                if _DECL.match(low):
                    for s in parse_decl(t):
                        s.module = module
                        if s.name in syms and syms[s.name].dummy:
                            s.dummy = True
                        syms[s.name] = s
                    continue
            except Unsupported as e:
                syms.setdefault("__bad__", []).append((st.where, str(e)))
                continue
        for n in syms.get("__save__", []):
            for k, v in syms.items():
                if isinstance(v, Sym) and (n == "*" or k == n):
                    v.save = True

    def _data(self, text, syms):
        body = text.strip()[4:].strip()
        for m in re.finditer(r"(\w+)\s*/([^/]*)/", body):
            name = m.group(1).lower()
            vals = [parse_expr(v) for v in _split_top(m.group(2), ",")]
            if name in syms:
                syms[name].data = vals
                syms[name].save = True

    def resolve(self, name, proc):
        """Symbol lookup: locals, the procedure's uses, the host module's
        variables and uses."""
        if proc is not None:
            if name in proc.syms and isinstance(proc.syms[name], Sym):
                return proc.syms[name]
            s = self._from_uses(name, proc.uses)
            if s:
                return s
            host = self.mods.get(proc.module)
        else:
            host = None
        if host:
            return self._mod_lookup(host, name, set())
        return None

    def _mod_lookup(self, mod, name, seen):
        if mod.name in seen:
            return None
        seen = seen | {mod.name}
        if name in mod.syms and isinstance(mod.syms[name], Sym):
            return mod.syms[name]
        return self._from_uses(name, mod.uses, seen)

    def _from_uses(self, name, uses, seen=frozenset()):
        for mn, only in uses:
            m = self.mods.get(mn)
            if m is None:
                continue
            if only is None:
                s = self._mod_lookup(m, name, set(seen))
                if s:
                    return s
            else:
                for local, remote in only:
                    if local == name:
                        return self._mod_lookup(m, remote, set(seen))
        return None

    def find_proc(self, name, proc):
        """A translated procedure visible from proc (by module)."""
        for m in self.mods.values():
            if name in m.procs and name in self.want:
                return m.procs[name]
        return None

    # ------------------------------------------------------------ constants
    def const(self, e, proc):
        """Evaluate a constant expression (parameters, kinds) -> python value."""
        if isinstance(e, Num):
            t = e.text.split("_")[0].lower().replace("d", "e")
            return float(t) if e.is_real else int(t)
        if isinstance(e, Bool):
            return e.v
        if isinstance(e, Str):
            return e.s
        if isinstance(e, Un):
            v = self.const(e.e, proc)
            return -v if e.op == "-" else (v if e.op in ("+", "()") else (not v))
        if isinstance(e, Bin):
            a, b = self.const(e.l, proc), self.const(e.r, proc)
            if e.op == "+":
                return a + b
            if e.op == "-":
                return a - b
            if e.op == "*":
                return a * b
            if e.op == "/":
                if isinstance(a, int) and isinstance(b, int):
                    q = abs(a) // abs(b)
                    return q if (a >= 0) == (b >= 0) else -q
                return a / b
            if e.op == "**":
                if isinstance(b, int):
                    return a ** b if isinstance(a, int) else _powi_py(float(a), b)
                return float(a) ** b
            if e.op == "//":
                return a + b
            raise Unsupported("const op " + e.op)
        if isinstance(e, Ref) and len(e.parts) == 1:
            name, args = e.parts[0]
            if args is None:
                s = self.resolve(name, proc)
                if s is None or not s.param:
                    raise Unsupported(f"not a constant: {name}")
                return self.param_value(s, proc)
            if name in ("kind", "selected_real_kind"):
                return 8 if name == "selected_real_kind" or self._lit_kind(args[0], proc) == "r" else 4
            if name == "selected_int_kind":
                return 4
            if name in ("real", "dble", "float"):
                return float(self.const(args[0], proc))
            if name == "int":
                return int(self.const(args[0], proc))
            if name in ("max", "min"):
                vals = [self.const(a, proc) for a in args]
                return max(vals) if name == "max" else min(vals)
            if name == "len":
                return len(self.const(args[0], proc))
            if name == "acos":
                import math
                return math.acos(self.const(args[0], proc))
        raise Unsupported("not a constant expression")

    def _lit_kind(self, e, proc):
        if isinstance(e, Num):
            return "r" if e.is_real else "i"
        if isinstance(e, Bool):
            return "l"
        return "r"

    def param_value(self, s, proc):
        if s.value is None:
            if s.init is None:
                raise Unsupported(f"parameter {s.name} without value")
            v = self.const(s.init, self._owner_proc(s))
            if s.base == "r":
                v = float(v)
            elif s.base == "i":
                v = int(v)
            s.value = v
        return s.value

    def _owner_proc(self, s):
        return None if s.module is None else Proc("__mod__", s.module, [], False, "", [], [])

    # ------------------------------------------------------------ C names and types
    def ctype(self, s):
        if s.base == "i" or s.base == "l":
            return "int"
        if s.base == "r":
            return "double"
        if s.base.startswith("t:"):
            return f"struct T_{s.base[2:]}"
        raise Unsupported(f"type of {s.name}")

    def esize(self, s):
        if s.base == "c":
            return self.clen(s)
        return f"(int)sizeof({self.ctype(s)})"

    def clen(self, s):
        if s.clen in (None, "*"):
            if s.init is not None and isinstance(s.init, Str):
                return len(s.init.s)
            if s.init is not None and isinstance(s.init, Cons):
                return max(len(x.s) for x in s.init.items)
            return 1
        try:
            return int(s.clen)
        except ValueError:
            return int(self.const(parse_expr(s.clen), self._owner_proc(s)))

    def gname(self, s):
        """C name of a module variable (registers its use)."""
        if not s.cname:
            s.cname = f"v_{s.module}__{s.name}"
        self.used_globals[s.cname] = s
        return s.cname

    # ------------------------------------------------------------ expressions
    def sym_code(self, s, ctx):
        """C lvalue of a scalar symbol or the RefArr of an array symbol."""
        if s.module is not None:
            return self.gname(s)
        if s.dummy:
            return f"(*a_{s.name})"
        return f"l_{s.name}"

    def gen(self, e, ctx):
        """-> (code, base) for a scalar (or elemental) expression."""
        if isinstance(e, Num):
            t = e.text.split("_")[0]
            if e.is_real:
                t = t.lower().replace("d", "e")
                if t.startswith("."):
                    t = "0" + t
                if "." not in t and "e" not in t:
                    t += ".0"
                return f"({t})", "r"
            return t, "i"
        if isinstance(e, Bool):
            return ("1" if e.v else "0"), "l"
        if isinstance(e, Str):
            lit = e.s.replace("\\", "\\\\").replace('"', '\\"')
            return f'((RefStr){{"{lit}", {len(e.s)}}})', "c"
        if isinstance(e, Un):
            if e.op == "()":
                c, b = self.gen(e.e, ctx)
                return (c if b == "c" else f"({c})"), b
            c, b = self.gen(e.e, ctx)
            if e.op == ".not.":
                return f"(!{c})", "l"
            return (f"(-{c})" if e.op == "-" else c), b
        if isinstance(e, Bin):
            return self.gen_bin(e, ctx)
        if isinstance(e, Ref):
            return self.gen_ref(e, ctx)
        if isinstance(e, Cons):
            raise Unsupported("array constructor in an expression")
        raise Unsupported(f"expression {type(e).__name__}")

    def conv(self, code, frm, to):
        if frm == to or to is None:
            return code
        if to == "r" and frm == "i":
            return f"((double){code})"
        if to == "i" and frm == "r":
            return f"((int){code})"
        if to == "l" and frm in ("i", "l"):
            return code
        if to == "i" and frm == "l":
            return code
        raise Unsupported(f"conversion {frm}->{to}")

    def gen_bin(self, e, ctx):
        op = e.op
        if op in (".and.", ".or."):
            a, _ = self.gen(e.l, ctx)
            b, _ = self.gen(e.r, ctx)
            return f"({a} {'&&' if op == '.and.' else '||'} {b})", "l"
        if op in (".eqv.", ".neqv."):
            a, _ = self.gen(e.l, ctx)
            b, _ = self.gen(e.r, ctx)
            return f"((!!{a}) {'==' if op == '.eqv.' else '!='} (!!{b}))", "l"
        if op == "**":
            return self.gen_pow(e, ctx)
        if op == "//":
            raise Unsupported("string concatenation")
        a, ta = self.gen(e.l, ctx)
        b, tb = self.gen(e.r, ctx)
        if op in ("==", "!=", "<", "<=", ">", ">="):
            if ta == "c" or tb == "c":
                if op not in ("==", "!="):
                    raise Unsupported("string ordering")
                return f"({'' if op == '==' else '!'}ref_streq({a}, {b}))", "l"
            if ta == "r" or tb == "r":
                a, b = self.conv(a, ta, "r"), self.conv(b, tb, "r")
            return f"({a} {op} {b})", "l"
        if ta == "r" or tb == "r":
            return f"({self.conv(a, ta, 'r')} {op} {self.conv(b, tb, 'r')})", "r"
        if ta == "i" and tb == "i":
            return f"({a} {op} {b})", "i"
        raise Unsupported(f"operands of {op}")

    def gen_pow(self, e, ctx):
        a, ta = self.gen(e.l, ctx)
        n = None
        try:
            n = self.const(e.r, ctx.proc)
        except Unsupported:
            n = None
        if isinstance(n, int):
            if ta == "i":
                return f"ref_ipow({a}, {n})", "i"
            if n == 0:
                return "(1.0)", "r"
            if abs(n) == 1:
                return (f"({a})" if n > 0 else f"(1.0 / ({a}))"), "r"
            if abs(n) not in _POWI:
                return f"ref_powi({a}, {n})", "r"
            v = ctx.newtmp("_pb")
            chain = _powi_chain(v, abs(n))
            body = chain if n > 0 else f"1.0 / {chain}"
            return f"({{ const double {v} = {a}; {body}; }})", "r"
        b, tb = self.gen(e.r, ctx)
        if tb == "i":
            if ta == "i":
                return f"ref_ipow({a}, {b})", "i"
            return f"ref_powi({a}, {b})", "r"
        return f"pow({self.conv(a, ta, 'r')}, {b})", "r"

    # array element / section handling ------------------------------------
    def elem_index(self, arr, s, args, ctx, where):
        """Offset expression of an element (args scalar or sections mapped
        onto the elemental loops)."""
        r = s.rank
        if args is None:
            args = [Rng(None, None)] * r
        if len(args) != r:
            raise Unsupported(f"rank of {s.name}")
        idx, k = [], 0
        for d, a in enumerate(args):
            if isinstance(a, Rng):
                if ctx.loops is None or k >= len(ctx.loops):
                    raise Unsupported(f"array section of {s.name} outside an array assignment")
                if a.st is not None:
                    raise Unsupported("strided section")
                lo = f"{arr}.lb[{d}]" if a.lo is None else self.conv(*self.gen(a.lo, ctx.scalar()), "i")
                lv, llo = ctx.loops[k]
                idx.append(f"({lo} + ({lv} - {llo}))")
                k += 1
            elif isinstance(a, Kw):
                raise Unsupported("keyword subscript")
            else:
                c, t = self.gen(a, ctx.scalar())
                idx.append(self.conv(c, t, "i"))
        if ctx.loops is not None and k and k != len(ctx.loops):
            raise Unsupported(f"section rank of {s.name}")
        w = where.replace('"', "'")
        idx = [f'RC({arr}, {d}, {x}, "{w}")' for d, x in enumerate(idx)]
        return f"ref_o{r}(&{arr}, {', '.join(idx)})" if r > 1 else f"({idx[0]} - {arr}.lb[0])"

    def has_section(self, args):
        return args is not None and any(isinstance(a, Rng) for a in args)

    def gen_ref(self, e, ctx):
        name, args = e.parts[0]
        s = self.resolve(name, ctx.proc)
        if s is None or (s.base == "c" and False):
            if len(e.parts) == 1:
                return self.gen_call(name, args or [], ctx)
            raise Unsupported(f"unknown name {name}")
        if s.param and s.rank == 0:
            v = self.param_value(s, ctx.proc)
            if s.base == "r":
                return f"({float(v).hex()})", "r"
            if s.base in ("i", "l"):
                return str(int(v)), s.base
            if s.base == "c":
                lit = v.replace('"', '\\"')
                return f'((RefStr){{"{lit}", {self.clen(s) if s.clen not in (None, "*") else len(v)}}})', "c"
        code, base, sym = self._ref_chain(e, ctx)
        return code, base

    def _ref_chain(self, e, ctx):
        """Walk name(args)%field(args)... -> (code, base, sym of last)."""
        name, args = e.parts[0]
        s = self.resolve(name, ctx.proc)
        code = self.sym_code(s, ctx)
        cur, cur_sym = code, s
        for pi, (nm, ag) in enumerate(e.parts):
            if pi > 0:
                tdef = self.types.get(cur_sym.base[2:]) if cur_sym.base.startswith("t:") else None
                if tdef is None or nm not in tdef.fields:
                    raise Unsupported(f"component {nm}")
                cur_sym = tdef.fields[nm]
                cur = f"{cur}.{nm}"
            if cur_sym.rank > 0:
                if ag is None and ctx.loops is None:
                    return cur, "arr:" + cur_sym.base, cur_sym
                off = self.elem_index(cur, cur_sym, ag, ctx, ctx.where)
                if cur_sym.base == "c":
                    ln = self.clen(cur_sym)
                    cur = f"((RefStr){{(char*){cur}.p + (long){ln} * {off}, {ln}}})"
                    if pi != len(e.parts) - 1:
                        raise Unsupported("component of a character")
                    return cur, "c", cur_sym
                cur = f"(({self.ctype(cur_sym)}*){cur}.p)[{off}]"
            else:
                if ag is not None:
                    if cur_sym.base == "c":
                        raise Unsupported("substring")
                    raise Unsupported(f"subscript on scalar {nm}")
                if cur_sym.base == "c":
                    ln = self.clen(cur_sym)
                    if pi != len(e.parts) - 1:
                        raise Unsupported("component of a character")
                    return f"((RefStr){{{cur}, {ln}}})", "c", cur_sym
        base = cur_sym.base
        return cur, base, cur_sym

    def gen_call(self, name, args, ctx):
        """Function call: a translated user function, else an intrinsic."""
        up = self.find_proc(name, ctx.proc)
        if up is not None and up.is_func:
            return self.gen_user_call(up, args, ctx)
        if name not in _INTRINSIC:
            raise Unsupported(f"function {name}")
        kw = {a.name: a.e for a in args if isinstance(a, Kw)}
        pos = [a for a in args if not isinstance(a, Kw)]
        sc = ctx.scalar() if name in ("size", "allocated", "minval", "maxval", "sum", "lbound", "ubound") else ctx
        if name in ("abs", "dabs"):
            c, t = self.gen(pos[0], ctx)
            return (f"fabs({c})" if t == "r" else f"abs({c})"), t
        if name in ("max", "min", "dmax1", "dmin1", "amax1", "amin1"):
            vals = [self.gen(a, ctx) for a in pos]
            isr = any(t == "r" for _, t in vals)
            f = ("ref_maxd" if isr else "ref_maxi") if name.startswith(("max", "dmax", "amax")) else \
                ("ref_mind" if isr else "ref_mini")
            acc = self.conv(vals[0][0], vals[0][1], "r" if isr else "i")
            for c, t in vals[1:]:
                acc = f"{f}({acc}, {self.conv(c, t, 'r' if isr else 'i')})"
            return acc, ("r" if isr else "i")
        if name in ("exp", "log", "log10", "sqrt", "sin", "cos", "tan", "asin", "acos", "atan", "sinh", "cosh",
                    "tanh", "dsqrt", "dexp", "dlog", "dlog10"):
            c, t = self.gen(pos[0], ctx)
            fn = {"dsqrt": "sqrt", "dexp": "exp", "dlog": "log", "dlog10": "log10"}.get(name, name)
            return f"{fn}({self.conv(c, t, 'r')})", "r"
        if name == "atan2":
            a, ta = self.gen(pos[0], ctx)
            b, tb = self.gen(pos[1], ctx)
            return f"atan2({self.conv(a, ta, 'r')}, {self.conv(b, tb, 'r')})", "r"
        if name in ("real", "dble", "float"):
            c, t = self.gen(pos[0], ctx)
            return self.conv(c, t, "r"), "r"
        if name == "int":
            c, t = self.gen(pos[0], ctx)
            return self.conv(c, t, "i"), "i"
        if name == "nint":
            c, t = self.gen(pos[0], ctx)
            return f"ref_nint({c})", "i"
        if name in ("floor", "ceiling"):
            c, t = self.gen(pos[0], ctx)
            return f"((int){name[:5] if name == 'floor' else 'ceil'}({c}))", "i"
        if name == "mod":
            a, ta = self.gen(pos[0], ctx)
            b, tb = self.gen(pos[1], ctx)
            if ta == "i" and tb == "i":
                return f"({a} % {b})", "i"
            return f"fmod({self.conv(a, ta, 'r')}, {self.conv(b, tb, 'r')})", "r"
        if name == "sign":
            a, ta = self.gen(pos[0], ctx)
            b, tb = self.gen(pos[1], ctx)
            if ta == "i":
                return f"ref_signi({a}, {b})", "i"
            return f"ref_signd({a}, {self.conv(b, tb, 'r')})", "r"
        if name in ("huge", "tiny", "epsilon"):
            _, t = self.gen(pos[0], ctx)
            if t == "i":
                return "INT_MAX", "i"
            return {"huge": "DBL_MAX", "tiny": "DBL_MIN", "epsilon": "DBL_EPSILON"}[name], "r"
        if name == "merge":
            a, ta = self.gen(pos[0], ctx)
            b, tb = self.gen(pos[1], ctx)
            m, _ = self.gen(pos[2], ctx)
            return f"(({m}) ? ({a}) : ({b}))", ta
        if name == "trim":
            c, t = self.gen(pos[0], ctx)
            return f"ref_trim({c})", "c"
        if name in ("kind", "selected_int_kind", "selected_real_kind"):
            return str(self.const(Ref([(name, args)]), ctx.proc)), "i"
        if name in ("allocated", "size", "lbound", "ubound"):
            arr, sym = self._whole_array(pos[0], ctx)
            if name == "allocated":
                return f"({arr}.p != NULL)", "l"
            dim = kw.get("dim", pos[1] if len(pos) > 1 else None)
            if name == "size":
                if dim is None:
                    return f"((int)ref_size(&{arr}))", "i"
                d, _ = self.gen(dim, ctx)
                return f"((int)({arr}.ub[({d}) - 1] - {arr}.lb[({d}) - 1] + 1))", "i"
            if dim is None:
                raise Unsupported("bound without dim")
            d, _ = self.gen(dim, ctx)
            return f"((int){arr}.{'lb' if name == 'lbound' else 'ub'}[({d}) - 1])", "i"
        if name in ("minval", "maxval", "sum"):
            if "mask" in kw or len(pos) > 1:
                raise Unsupported(f"{name} with mask/dim")
            return self.gen_reduce(name, pos[0], ctx)
        raise Unsupported(f"intrinsic {name}")

    def gen_user_call(self, p, args, ctx):
        """A translated function: arguments by reference (temporaries for
        expressions) inside a statement expression."""
        self.prepare_proc(p)
        self.ensure_proc(p)
        if len(args) != len(p.args):
            raise Unsupported(f"argument count of {p.name}")
        pre, cargs = [], []
        for dn, a in zip(p.args, args):
            ds = p.syms.get(dn)
            if ds is None or isinstance(a, Kw) or ds.rank or ds.base not in ("i", "r", "l"):
                raise Unsupported(f"argument {dn} of {p.name}")
            c, t = self.gen(a, ctx.scalar())
            v = ctx.newtmp("_fa")
            pre.append(f"{self.ctype(ds)} {v} = {self.conv(c, t, ds.base)};")
            cargs.append(f"&{v}")
        r = p.syms.get(p.result)
        if r is None:
            raise Unsupported(f"result of {p.name}")
        return f"({{ {' '.join(pre)} {self.proc_cname(p)}({', '.join(cargs)}); }})", r.base

    def _whole_array(self, e, ctx):
        if not isinstance(e, Ref):
            raise Unsupported("array argument")
        sub = ctx.scalar()
        code, base, sym = self._ref_chain_noelem(e, sub)
        return code, sym

    def _ref_chain_noelem(self, e, ctx):
        """The RefArr of name or name(i)%field (last part unsubscripted)."""
        last_name, last_args = e.parts[-1]
        if last_args is not None:
            raise Unsupported("subscripted array argument")
        if len(e.parts) == 1:
            s = self.resolve(last_name, ctx.proc)
            if s is None or s.rank == 0:
                raise Unsupported("not an array")
            return self.sym_code(s, ctx), s.base, s
        head = Ref(e.parts[:-1])
        code, base, sym = self._ref_chain(head, ctx)
        tdef = self.types.get(base[2:]) if base.startswith("t:") else None
        if tdef is None or last_name not in tdef.fields:
            raise Unsupported("component")
        f = tdef.fields[last_name]
        return f"{code}.{last_name}", f.base, f

    def gen_reduce(self, name, e, ctx):
        if not isinstance(e, Ref) or len(e.parts) != 1:
            raise Unsupported("reduction operand")
        nm, args = e.parts[0]
        s = self.resolve(nm, ctx.proc)
        if s is None or s.rank == 0:
            raise Unsupported("reduction of a scalar")
        arr = self.sym_code(s, ctx)
        if args is None:
            args = [Rng(None, None)] * s.rank
        loops, hdr, k = [], [], 0
        for d, a in enumerate(args):
            if isinstance(a, Rng):
                v = ctx.newtmp("_r")
                lo = f"{arr}.lb[{d}]" if a.lo is None else self.conv(*self.gen(a.lo, ctx.scalar()), "i")
                hi = f"{arr}.ub[{d}]" if a.hi is None else self.conv(*self.gen(a.hi, ctx.scalar()), "i")
                vlo = ctx.newtmp("_rl")
                hdr.append(f"for (long {v} = {lo}, {vlo} = {v}; {v} <= {hi}; ++{v})")
                loops.append((v, vlo))
                k += 1
        sub = ctx.with_loops(loops)
        el, t = self.gen(e, sub)
        acc = ctx.newtmp("_acc")
        ct = "double" if t == "r" else "int"
        init = {"sum": "0", "minval": "DBL_MAX" if t == "r" else "INT_MAX",
                "maxval": "-DBL_MAX" if t == "r" else "INT_MIN"}[name]
        upd = {"sum": f"{acc} = {acc} + ({el});",
               "minval": f"{{ {ct} _v = ({el}); if (_v < {acc}) {acc} = _v; }}",
               "maxval": f"{{ {ct} _v = ({el}); if (_v > {acc}) {acc} = _v; }}"}[name]
        loops_c = " ".join(reversed(hdr))
        return f"({{ {ct} {acc} = {init}; {loops_c} {upd} {acc}; }})", t

    # ------------------------------------------------------------ statements
    _END_DO = re.compile(r"^end\s*do\b")
    _END_IF = re.compile(r"^end\s*if\b")
    _ELSE_IF = re.compile(r"^else\s*if\s*\(")
    _ELSE = re.compile(r"^else\s*$")
    _END_SEL = re.compile(r"^end\s*select\b")
    _CASE = re.compile(r"^case\s*(\(|default\b)")
    _DO = re.compile(r"^(?:\w+\s*:\s*)?do(\s+\w+\s*=.*|\s+while\s*\(.*|\s*)$")
    _IF_THEN = re.compile(r"^(?:\w+\s*:\s*)?if\s*\(")
    _SELECT = re.compile(r"^(?:\w+\s*:\s*)?select\s*case\s*\(")
    _WHERE = re.compile(r"^where\s*\(")

    @staticmethod
    def _paren(text, start):
        """(inside, index after) of the parenthesised group at text[start]."""
        depth, q = 0, None
        for j in range(start, len(text)):
            ch = text[j]
            if q:
                if ch == q:
                    q = None
                continue
            if ch in "'\"":
                q = ch
            elif ch == "(":
                depth += 1
            elif ch == ")":
                depth -= 1
                if depth == 0:
                    return text[start + 1:j], j + 1
        raise Unsupported("unbalanced parentheses")

    def _is_if_then(self, text):
        low = text.lower()
        if not self._IF_THEN.match(low):
            return False
        k = low.index("(")
        _, j = self._paren(text, k)
        return low[j:].strip() == "then"

    def _skip(self, stmts, i, opener, closer):
        """Index after the statement closing the construct opened at i."""
        depth = 0
        while i < len(stmts):
            low = stmts[i].text.lower().strip()
            if stmts[i].omp:
                i += 1
                continue
            if opener(low):
                depth += 1
            elif closer(low):
                depth -= 1
                if depth == 0:
                    return i + 1
            i += 1
        raise Unsupported("unterminated construct")

    def _fail(self, out, ind, st, why):
        msg = f"{st.where}: {why}".replace("\\", "/").replace('"', "'")[:300]
        out.append(f'{ind}ref_fail("{msg}");')

    def block(self, stmts, i, ctx, out, ind, end):
        omp = None
        while i < len(stmts):
            st = stmts[i]
            if st.omp:
                if re.match(r"parallel\s+do", st.omp):
                    omp = st.omp
                i += 1
                continue
            low = st.text.lower().strip()
            if end(low):
                return i
            ctx.where = st.where
            i = self.stmt(stmts, i, ctx, out, ind, omp)
            omp = None
        return i

    def stmt(self, stmts, i, ctx, out, ind, omp=None):
        st = stmts[i]
        text = st.text.strip()
        low = text.lower()
        is_do = lambda l: bool(self._DO.match(l)) and not self._END_DO.match(l)
        if self._DO.match(low) and not self._END_DO.match(low):
            try:
                return self.do_loop(stmts, i, ctx, out, ind, omp)
            except Unsupported as e:
                j = self._skip(stmts, i, is_do, lambda l: bool(self._END_DO.match(l)))
                self._fail(out, ind, st, str(e))
                return j
        if self._is_if_then(text):
            return self.if_block(stmts, i, ctx, out, ind)
        if self._SELECT.match(low):
            try:
                return self.select_block(stmts, i, ctx, out, ind)
            except Unsupported as e:
                j = self._skip(stmts, i, lambda l: bool(self._SELECT.match(l)), lambda l: bool(self._END_SEL.match(l)))
                self._fail(out, ind, st, str(e))
                return j
        if self._WHERE.match(low) and not re.match(r"^where\s*\(.*\)\s*\w.*=", low):
            j = self._skip(stmts, i, lambda l: bool(self._WHERE.match(l)), lambda l: bool(re.match(r"^end\s*where", l)))
            self._fail(out, ind, st, "where block")
            return j
        try:
            self.simple(text, ctx, out, ind, st)
        except Unsupported as e:
            self._fail(out, ind, st, str(e))
        return i + 1

    def do_loop(self, stmts, i, ctx, out, ind, omp):
        st = stmts[i]
        text = st.text.strip()
        m = re.match(r"^(?:\w+\s*:\s*)?do\s+(\w+)\s*=\s*(.*)$", text, re.I)
        body_end = lambda l: bool(self._END_DO.match(l))
        if m:
            var = m.group(1).lower()
            parts = _split_top(m.group(2), ",")
            if len(parts) not in (2, 3):
                raise Unsupported("do bounds")
            s = self.resolve(var, ctx.proc)
            if s is None or s.base != "i" or s.rank:
                raise Unsupported("do variable")
            vc = self.sym_code(s, ctx)
            lo = self.conv(*self.gen(parse_expr(parts[0]), ctx), "i")
            hi = self.conv(*self.gen(parse_expr(parts[1]), ctx), "i")
            step = 1
            if len(parts) == 3:
                try:
                    step = self.const(parse_expr(parts[2]), ctx.proc)
                except Unsupported:
                    raise Unsupported("non-constant do step")
            h = ctx.newtmp("_hi")
            out.append(f"{ind}{{ const int {h} = {hi};")
            if omp:
                if s.dummy or s.module is not None:
                    raise Unsupported("parallel loop over a non-local variable")
                out.append(f"{ind}#pragma omp parallel for")
            cmp = "<=" if step > 0 else ">="
            out.append(f"{ind}for ({vc} = {lo}; {vc} {cmp} {h}; {vc} += {step}) {{")
            if omp:
                out.append(f"{ind}  ref_in_parallel = 1;")
            j = self.block(stmts, i + 1, ctx, out, ind + "  ", body_end)
            out.append(f"{ind}}}")
            if omp:
                out.append(f"{ind}ref_in_parallel = 0; if (ref_errset) longjmp(ref_jb, 1);")
            out.append(f"{ind}}}")
            return j + 1
        m = re.match(r"^(?:\w+\s*:\s*)?do\s+while\s*(\(.*\))\s*$", text, re.I)
        if m:
            inner, _ = self._paren(m.group(1), 0)
            c, _ = self.gen(parse_expr(inner), ctx)
            out.append(f"{ind}while ({c}) {{")
            j = self.block(stmts, i + 1, ctx, out, ind + "  ", body_end)
            out.append(f"{ind}}}")
            return j + 1
        raise Unsupported("do form")

    def if_block(self, stmts, i, ctx, out, ind):
        st = stmts[i]
        text = st.text.strip()
        is_open = lambda l: self._is_if_then(l)
        is_close = lambda l: bool(self._END_IF.match(l))
        inner, _ = self._paren(text, text.index("("))
        try:
            c, _ = self.gen(parse_expr(inner), ctx)
        except Unsupported as e:
            j = self._skip(stmts, i, is_open, is_close)
            self._fail(out, ind, st, str(e))
            return j
        out.append(f"{ind}if ({c}) {{")
        stop = lambda l: bool(self._END_IF.match(l) or self._ELSE_IF.match(l) or self._ELSE.match(l))
        j = self.block(stmts, i + 1, ctx, out, ind + "  ", stop)
        while j < len(stmts):
            t = stmts[j].text.strip()
            low = t.lower()
            ctx.where = stmts[j].where
            if self._END_IF.match(low):
                out.append(f"{ind}}}")
                return j + 1
            if self._ELSE_IF.match(low):
                inner, _ = self._paren(t, t.index("("))
                try:
                    c, _ = self.gen(parse_expr(inner), ctx)
                except Unsupported as e:
                    out.append(f"{ind}}} else {{")
                    self._fail(out, ind + "  ", stmts[j], str(e))
                    # skip to the matching end if
                    depth, k = 1, j + 1
                    while k < len(stmts):
                        lw = stmts[k].text.lower().strip()
                        if not stmts[k].omp and self._is_if_then(stmts[k].text.strip()):
                            depth += 1
                        elif not stmts[k].omp and self._END_IF.match(lw):
                            depth -= 1
                            if depth == 0:
                                break
                        k += 1
                    out.append(f"{ind}}}")
                    return k + 1
                out.append(f"{ind}}} else if ({c}) {{")
            else:
                out.append(f"{ind}}} else {{")
            j = self.block(stmts, j + 1, ctx, out, ind + "  ", stop)
        raise Unsupported("unterminated if")

    def select_block(self, stmts, i, ctx, out, ind):
        st = stmts[i]
        text = st.text.strip()
        inner, _ = self._paren(text, text.index("("))
        sel, tb = self.gen(parse_expr(inner), ctx)
        v = ctx.newtmp("_sel")
        out.append(f"{ind}{{ const {'RefStr' if tb == 'c' else ('double' if tb == 'r' else 'int')} {v} = {sel};")
        j = i + 1
        cases = []   # (cond or None for default, lines)
        stop = lambda l: bool(self._CASE.match(l) or self._END_SEL.match(l))
        while j < len(stmts) and not (stmts[j].omp or self._CASE.match(stmts[j].text.lower().strip())):
            j += 1
        while j < len(stmts):
            t = stmts[j].text.strip()
            low = t.lower()
            if self._END_SEL.match(low):
                break
            body = []
            if re.match(r"^case\s+default", low):
                cond = None
            else:
                items, _ = self._paren(t, t.index("("))
                conds = []
                for it in _split_top(items, ","):
                    rng = _split_top(it, ":")
                    if len(rng) == 1:
                        c, t2 = self.gen(parse_expr(it), ctx)
                        conds.append(f"ref_streq({v}, {c})" if tb == "c" else f"({v} == {c})")
                    else:
                        if tb == "c":
                            raise Unsupported("character case range")
                        cs = []
                        if rng[0].strip():
                            cs.append(f"({v} >= {self.gen(parse_expr(rng[0]), ctx)[0]})")
                        if rng[1].strip():
                            cs.append(f"({v} <= {self.gen(parse_expr(rng[1]), ctx)[0]})")
                        conds.append("(" + " && ".join(cs or ["1"]) + ")")
                cond = " || ".join(conds)
            j = self.block(stmts, j + 1, ctx, body, ind + "  ", stop)
            cases.append((cond, body))
        first = True
        default = None
        for cond, body in cases:
            if cond is None:
                default = body
                continue
            out.append(f"{ind}{'if' if first else '} else if'} ({cond}) {{")
            out.extend(body)
            first = False
        if default is not None:
            out.append(f"{ind}{'{' if first else '} else {'}")
            out.extend(default)
            first = False
        if not first:
            out.append(f"{ind}}}")
        out.append(f"{ind}}}")
        return j + 1

    def simple(self, text, ctx, out, ind, st):
        low = text.lower()
        if _IO.match(low):
            return
        if re.match(r"^if\s*\(", low):
            inner, j = self._paren(text, text.index("("))
            rest = text[j:].strip()
            c, _ = self.gen(parse_expr(inner), ctx)
            sub = []
            try:
                self.simple(rest, ctx, sub, ind + "  ", st)
            except Unsupported as e:
                sub = []
                self._fail(sub, ind + "  ", st, str(e))
            out.append(f"{ind}if ({c}) {{")
            out.extend(sub)
            out.append(f"{ind}}}")
            return
        if re.match(r"^call\b", low):
            return self.call(text, ctx, out, ind)
        if re.match(r"^return\s*$", low):
            out.append(f"{ind}goto _ret;")
            return
        if re.match(r"^cycle\s*$", low):
            out.append(f"{ind}continue;")
            return
        if re.match(r"^exit\s*$", low):
            out.append(f"{ind}break;")
            return
        if re.match(r"^continue\s*$", low):
            return
        if re.match(r"^stop\b", low) or re.match(r"^error\s+stop\b", low):
            self._fail(out, ind, st, "stop")
            return
        if re.match(r"^(de)?allocate\s*\(", low):
            return self.alloc_stmt(text, ctx, out, ind)
        idx = _find_assign(text)
        if idx > 0:
            return self.assign(text[:idx], text[idx + 1:], ctx, out, ind)
        raise Unsupported(f"statement {text[:40]!r}")

    def call(self, text, ctx, out, ind):
        m = re.match(r"^call\s+(\w+)\s*(\(.*\))?\s*$", text, re.I)
        if not m:
            raise Unsupported("call")
        name = m.group(1).lower()
        p = self.find_proc(name, ctx.proc)
        if p is None:
            out.append(f'{ind}ref_stub("{name}");')
            return
        args = Parser(tokenize(m.group(2))).arglist() if m.group(2) else []
        self.prepare_proc(p)
        self.ensure_proc(p)
        pre, cargs = [], []
        if len(args) != len(p.args):
            raise Unsupported(f"argument count of {name}")
        for dn, a in zip(p.args, args):
            ds = p.syms.get(dn)
            if ds is None:
                raise Unsupported(f"undeclared dummy {dn}")
            if isinstance(a, Kw):
                raise Unsupported("keyword argument")
            if ds.rank > 0:
                arr, sym = self._whole_array(a, ctx)
                cargs.append(f"&{arr}")
                continue
            if isinstance(a, Ref):
                s = self.resolve(a.parts[0][0], ctx.proc)
                if s is not None and not s.param and ds.base != "c":
                    code, base, sym = self._ref_chain(a, ctx.scalar())
                    if base == ds.base:
                        cargs.append(f"&({code})")
                        continue
            c, t = self.gen(a, ctx.scalar())
            if ds.base == "c":
                raise Unsupported("character argument")
            v = ctx.newtmp("_a")
            pre.append(f"{self.ctype(ds)} {v} = {self.conv(c, t, ds.base)};")
            cargs.append(f"&{v}")
        out.append(f"{ind}{{ {' '.join(pre)} {self.proc_cname(p)}({', '.join(cargs)}); }}")

    def alloc_stmt(self, text, ctx, out, ind):
        dealloc = text.lower().startswith("de")
        inner, _ = self._paren(text, text.index("("))
        for it in _split_top(inner, ","):
            it = it.strip()
            if re.match(r"^(stat|errmsg|source|mold)\s*=", it, re.I):
                continue
            e = Parser(tokenize(it)).primary()
            if not isinstance(e, Ref):
                raise Unsupported("allocate object")
            if dealloc:
                arr, sym = self._whole_array(e, ctx)
                out.append(f"{ind}ref_dealloc(&{arr});")
                continue
            last, dims = e.parts[-1]
            if dims is None:
                raise Unsupported("allocate without shape")
            arr, sym = self._whole_array(Ref(e.parts[:-1] + [(last, None)]), ctx)
            lbs, ubs = [], []
            for d in dims:
                if isinstance(d, Rng):
                    lbs.append(self.conv(*self.gen(d.lo, ctx.scalar()), "i"))
                    ubs.append(self.conv(*self.gen(d.hi, ctx.scalar()), "i"))
                else:
                    lbs.append("1")
                    ubs.append(self.conv(*self.gen(d, ctx.scalar()), "i"))
            w = ctx.where
            out.append(f"{ind}{{ const long _lb[] = {{{', '.join(lbs)}}}, _ub[] = {{{', '.join(ubs)}}}; "
                       f'ref_alloc(&{arr}, {self.esize(sym)}, {len(dims)}, _lb, _ub, "{w}: allocated twice"); }}')
            if sym.base == "c":
                out.append(f"{ind}memset({arr}.p, ' ', (size_t)ref_size(&{arr}) * {arr}.esz);")

    def assign(self, lhs_t, rhs_t, ctx, out, ind):
        lp = Parser(tokenize(lhs_t))
        lhs = lp.primary()
        if not lp.done() or not isinstance(lhs, Ref):
            raise Unsupported("assignment target")
        rhs = parse_expr(rhs_t)
        name, args = lhs.parts[0]
        s = self.resolve(name, ctx.proc)
        if s is None:
            raise Unsupported(f"unknown variable {name}")
        if s.param:
            raise Unsupported("assignment to a parameter")
        # array assignment: a single-part reference to an array, whole or sectioned
        if len(lhs.parts) == 1 and s.rank > 0 and (args is None or self.has_section(args)):
            if s.base == "c":
                raise Unsupported("character array assignment")
            arr = self.sym_code(s, ctx)
            if args is None:
                args = [Rng(None, None)] * s.rank
            loops, decl, hdr = [], [], []
            for d, a in enumerate(args):
                if isinstance(a, Rng):
                    if a.st is not None:
                        raise Unsupported("strided section")
                    lo = f"{arr}.lb[{d}]" if a.lo is None else self.conv(*self.gen(a.lo, ctx.scalar()), "i")
                    hi = f"{arr}.ub[{d}]" if a.hi is None else self.conv(*self.gen(a.hi, ctx.scalar()), "i")
                    vlo, vhi, v = ctx.newtmp("_lo"), ctx.newtmp("_hi"), ctx.newtmp("_i")
                    decl.append(f"const long {vlo} = {lo}, {vhi} = {hi};")
                    hdr.append(f"for (long {v} = {vlo}; {v} <= {vhi}; ++{v})")
                    loops.append((v, vlo))
            ec = ctx.with_loops(loops)
            off = self.elem_index(arr, s, args, ec, ctx.where)
            rc, rt = self.gen(rhs, ec)
            if rt == "c" or rt.startswith("arr:"):
                raise Unsupported("array assignment operand")
            out.append(f"{ind}{{ {' '.join(decl)}")
            out.append(f"{ind}  {' '.join(reversed(hdr))}")
            out.append(f"{ind}    (({self.ctype(s)}*){arr}.p)[{off}] = {self.conv(rc, rt, s.base)};")
            out.append(f"{ind}}}")
            return
        code, base, sym = self._ref_chain(lhs, ctx.scalar())
        if base.startswith("arr:"):
            raise Unsupported("array component assignment")
        rc, rt = self.gen(rhs, ctx.scalar())
        if base == "c":
            out.append(f"{ind}{{ RefStr _d = {code}; ref_sassign((char*)_d.p, _d.n, {rc}); }}")
            return
        if base.startswith("t:"):
            if rt != base:
                raise Unsupported("derived-type assignment")
            out.append(f"{ind}{code} = {rc};")
            return
        out.append(f"{ind}{code} = {self.conv(rc, rt, base)};")

    # ------------------------------------------------------------ procedures
    def proc_cname(self, p):
        return f"f_{p.module}__{p.name}"

    def ensure_proc(self, p):
        if p.name not in self.translated:
            self.translated[p.name] = None
            self._todo.append(p)

    def proc_sig(self, p):
        parms = []
        for a in p.args:
            s = p.syms.get(a)
            if s is None:
                raise Unsupported(f"undeclared dummy {a} of {p.name}")
            parms.append(f"RefArr* a_{a}" if s.rank else f"{self.ctype(s)}* a_{a}")
        ret = "void"
        if p.is_func:
            r = p.syms.get(p.result)
            ret = self.ctype(r)
        return f"{ret} {self.proc_cname(p)}({', '.join(parms) or 'void'})"

    def prepare_proc(self, p):
        if getattr(p, "_prepared", False):
            return
        p._prepared = True
        self._spec(p, p.spec, p.syms, p.uses)
        for a in p.args:
            if a in p.syms:
                p.syms[a].dummy = True

    def translate_proc(self, p):
        self.prepare_proc(p)
        ctx = Ctx(self, p)
        lines, init, fin = [], [], []
        for name, s in p.syms.items():
            if not isinstance(s, Sym) or s.dummy or s.param and s.rank == 0:
                continue
            if p.is_func and name == p.result:
                lines.append(f"  {self.ctype(s)} l_{name} = 0;")
                continue
            st = "static " if (s.save or s.data or s.init is not None) else ""
            if s.rank == 0:
                if s.base == "c":
                    ln = self.clen(s)
                    iv = self.const(s.init, p) if s.init is not None else ""
                    lit = (iv + " " * ln)[:ln].replace('"', '\\"')
                    if st:
                        lines.append(f'  static char l_{name}[{ln}] = "{lit}";')
                    else:
                        lines.append(f"  char l_{name}[{ln}]; memset(l_{name}, ' ', {ln});")
                elif s.base.startswith("t:"):
                    lines.append(f"  {st}{self.ctype(s)} l_{name}; memset(&l_{name}, 0, sizeof l_{name});")
                else:
                    iv = "0"
                    if s.init is not None:
                        v = self.const(s.init, p)
                        iv = float(v).hex() if s.base == "r" else str(int(v))
                    lines.append(f"  {st}{self.ctype(s)} l_{name} = {iv};")
                continue
            lines.append(f"  {st}RefArr l_{name} = {{0}};")
            if s.alloc:
                if not st:
                    fin.append(f"  if (l_{name}.p) ref_dealloc(&l_{name});")
                continue
            lbs, ubs = [], []
            for lo, hi in s.dims:
                if hi is None:
                    raise Unsupported(f"assumed shape local {name}")
                lbs.append(self.conv(*self.gen(lo, ctx), "i"))
                ubs.append(self.conv(*self.gen(hi, ctx), "i"))
            a = (f"{{ const long _lb[] = {{{', '.join(lbs)}}}, _ub[] = {{{', '.join(ubs)}}}; "
                 f'ref_alloc(&l_{name}, {self.esize(s)}, {len(lbs)}, _lb, _ub, "{p.name}"); }}')
            vals = s.data or (s.init.items if isinstance(s.init, Cons) else None)
            fill = []
            if s.base == "c":
                fill.append(f"memset(l_{name}.p, ' ', (size_t)ref_size(&l_{name}) * l_{name}.esz);")
            if vals:
                for k, vv in enumerate(vals):
                    v = self.const(vv, p)
                    if s.base == "c":
                        ln = self.clen(s)
                        lit = (v + " " * ln)[:ln].replace('"', '\\"')
                        fill.append(f'memcpy((char*)l_{name}.p + {k * ln}, "{lit}", {ln});')
                    elif s.base == "r":
                        fill.append(f"((double*)l_{name}.p)[{k}] = {float(v).hex()};")
                    else:
                        fill.append(f"((int*)l_{name}.p)[{k}] = {int(v)};")
            if st:
                init.append(f"  if (!l_{name}.p) {{ {a} {' '.join(fill)} }}")
            else:
                init.append(f"  {a} {' '.join(fill)}")
                fin.append(f"  ref_dealloc(&l_{name});")
        body = []
        self.block(p.body, 0, ctx, body, "  ", lambda l: False)
        code = [self.proc_sig(p) + " {"] + lines + init + body + ["_ret:;"] + fin
        if p.is_func:
            code.append(f"  return l_{p.result};")
        code.append("}")
        return code

    # ------------------------------------------------------------ driver
    def run(self):
        self.setup()
        self._todo = []
        for name in self.want:
            p = self.find_proc(name, None)
            if p is None:
                raise SystemExit(f"procedure {name} not found")
            self.ensure_proc(p)
        bodies = []
        while self._todo:
            p = self._todo.pop(0)
            self.prepare_proc(p)
            try:
                bodies.append(self.translate_proc(p))
                self.translated[p.name] = self.proc_cname(p)
            except Unsupported as e:
                raise SystemExit(f"cannot translate {p.name}: {e}")
        return bodies

    def emit(self, bodies):
        out = [PRELUDE]
        # derived types used by globals and locals
        used_types = set()

        def need_type(tn, seen=None):
            if tn in used_types:
                return
            td = self.types.get(tn)
            if td is None:
                raise SystemExit(f"unknown type {tn}")
            for f in td.fields.values():
                if f.base.startswith("t:"):
                    need_type(f.base[2:])
            used_types.add(tn)
            tdefs.append(td)

        tdefs = []
        for s in list(self.used_globals.values()):
            if s.base.startswith("t:"):
                need_type(s.base[2:])
        for p in self.mods_procs():
            for s in p.syms.values():
                if isinstance(s, Sym) and s.base.startswith("t:"):
                    need_type(s.base[2:])
        for td in tdefs:
            out.append(f"struct T_{td.name} {{")
            for f in td.fields.values():
                if f.rank:
                    out.append(f"  RefArr {f.name};")
                elif f.base == "c":
                    out.append(f"  char {f.name}[{self.clen(f)}];")
                else:
                    out.append(f"  {self.ctype(f)} {f.name};")
            out.append("};")
        # globals
        ginit = []
        for cn, s in sorted(self.used_globals.items()):
            tls = "__thread " if s.tls else ""
            owner = self._owner_proc(s)
            if s.rank == 0:
                if s.base == "c":
                    ln = self.clen(s)
                    iv = self.const(s.init, owner) if s.init is not None else ""
                    lit = (iv + " " * ln)[:ln].replace('"', '\\"')
                    out.append(f"static {tls}char {cn}[{ln}];")
                    ginit.append(f'  memcpy({cn}, "{lit}", {ln});')
                elif s.base.startswith("t:"):
                    out.append(f"static {tls}{self.ctype(s)} {cn};")
                    ginit.append(f"  memset(&{cn}, 0, sizeof {cn});")
                else:
                    iv = "0"
                    if s.init is not None:
                        v = self.param_value(s, owner) if s.param else self.const(s.init, owner)
                        iv = float(v).hex() if s.base == "r" else str(int(v))
                    out.append(f"static {tls}{self.ctype(s)} {cn};")
                    ginit.append(f"  {cn} = {iv};")
                continue
            out.append(f"static {tls}RefArr {cn};")
            ginit.append(f"  if ({cn}.p) ref_dealloc(&{cn});")
            if s.alloc:
                continue
            lbs, ubs = [], []
            for lo, hi in s.dims:
                lbs.append(str(int(self.const(lo, owner))))
                ubs.append(str(int(self.const(hi, owner))))
            ginit.append(f"  {{ const long _lb[] = {{{', '.join(lbs)}}}, _ub[] = {{{', '.join(ubs)}}}; "
                         f'ref_alloc(&{cn}, {self.esize(s)}, {len(lbs)}, _lb, _ub, "{cn}"); }}')
            if s.base == "c":
                ginit.append(f"  memset({cn}.p, ' ', (size_t)ref_size(&{cn}) * {cn}.esz);")
            vals = s.data or (s.init.items if isinstance(s.init, Cons) else None)
            for k, vv in enumerate(vals or []):
                v = self.const(vv, owner)
                if s.base == "c":
                    ln = self.clen(s)
                    lit = (v + " " * ln)[:ln].replace('"', '\\"')
                    ginit.append(f'  memcpy((char*){cn}.p + {k * ln}, "{lit}", {ln});')
                elif s.base == "r":
                    ginit.append(f"  ((double*){cn}.p)[{k}] = {float(v).hex()};")
                else:
                    ginit.append(f"  ((int*){cn}.p)[{k}] = {int(v)};")
        # prototypes and bodies
        ps = [p for p in self.mods_procs() if self.translated.get(p.name)]
        for p in ps:
            out.append("static " + self.proc_sig(p) + ";")
        for b in bodies:
            out.append("static " + b[0])
            out.extend(b[1:])
        # exported API
        out.append("int ref_init(void) {")
        out.extend(ginit)
        out.append("  ref_errset = 0; ref_errbuf[0] = 0; ref_nstub = 0;")
        out.append("  memset(ref_stub_calls, 0, sizeof ref_stub_calls);")
        out.append("  return 0;\n}")
        out.append("void* ref_addr(const char* n, int* base, int* rank, int* esz) {")
        for cn, s in sorted(self.used_globals.items()):
            key = f"{s.module}::{s.name}"
            b = {"i": 0, "r": 1, "l": 2, "c": 3}.get(s.base, 4)
            es = self.esize(s) if not s.base.startswith("t:") else f"(int)sizeof({self.ctype(s)})"
            addr = cn if (s.base == "c" and s.rank == 0) else f"&{cn}"
            out.append(f'  if (!strcmp(n, "{key}")) {{ *base = {b}; *rank = {s.rank}; *esz = {es}; '
                       f"return (void*){addr}; }}")
        out.append("  return NULL;\n}")
        out.append("int ref_alloc_var(const char* n, int rank, const long* lb, const long* ub) {")
        out.append("  int b, r, e; RefArr* a = (RefArr*)ref_addr(n, &b, &r, &e);")
        out.append("  if (!a || r != rank || rank == 0) return -1;")
        out.append("  if (a->p) ref_dealloc(a);")
        out.append("  ref_errset = 0; if (setjmp(ref_jb)) return -1;")
        out.append('  ref_alloc(a, e, rank, lb, ub, n);')
        out.append("  if (b == 3) memset(a->p, ' ', (size_t)ref_size(a) * e);")
        out.append("  return 0;\n}")
        out.append("int ref_call(const char* n, int na, int* args) {")
        out.append("  int a[8] = {0};")
        out.append("  for (int i = 0; i < na && i < 8; ++i) a[i] = args[i];")
        out.append("  ref_errset = 0; ref_errbuf[0] = 0;")
        out.append("  if (setjmp(ref_jb)) return -1;")
        for p in ps:
            if p.is_func:
                continue
            if not all((p.syms[a].base == "i" and p.syms[a].rank == 0) for a in p.args):
                continue
            ca = ", ".join(f"&a[{k}]" for k in range(len(p.args)))
            out.append(f'  if (!strcmp(n, "{p.name}")) {{ if (na != {len(p.args)}) return -3; '
                       f"{self.proc_cname(p)}({ca}); for (int i = 0; i < na && i < 8; ++i) args[i] = a[i]; "
                       f"return ref_errset ? -1 : 0; }}")
        out.append("  return -2;\n}")
        out.append("const char* ref_error(void) { return ref_errbuf; }")
        out.append("int ref_nstubs(void) { return ref_nstub; }")
        out.append("const char* ref_stub_name(int i) { return i >= 0 && i < ref_nstub ? ref_stub_names[i] : \"\"; }")
        out.append("long ref_stub_count(int i) { return i >= 0 && i < ref_nstub ? ref_stub_calls[i] : 0; }")
        out.append("void ref_stub_reset(void) { ref_nstub = 0; memset(ref_stub_calls, 0, sizeof ref_stub_calls); }")
        out.append("void ref_threads(int n) {\n#ifdef _OPENMP\n  omp_set_num_threads(n > 0 ? n : 1);\n#else\n"
                   "  (void)n;\n#endif\n}")
        return "\n".join(out) + "\n"

    def mods_procs(self):
        for m in self.mods.values():
            for p in m.procs.values():
                yield p


# ---------------------------------------------------------------- command line
# Files holding the routines of the kinetic step, their modules, and the
# helper modules they use, relative to the reference's tree.
REF_FILES = ["src/nrtype.f90", "share/Library/src/ModNumConst.f90", "share/Library/src/ModTimeConvert.f90",
             "src/ModRamGrids.f90", "src/ModRamMain.f90", "src/ModRamParams.f90", "src/ModRamTiming.f90",
             "src/ModRamConst.f90", "src/ModRamSpecies.f90", "src/ModRamVariables.f90", "src/ModRamDrift.f90",
             "src/ModRamLoss.f90", "src/ModRamRun.f90", "src/ModRamInit.f90", "src/ModRamFunctions.f90",
             "src/ModRamWPI.f90"]
REF_PROCS = ["definespecies", "driftend", "driftpara", "driftr", "driftp", "drifte", "driftmu", "cepara",
             "charexchange", "atmol", "ram_run", "sumrc", "anisch", "arrays", "acosd", "asind", "cosd", "sind",
             "ram_sum_pressure", "wpadif", "flcscatter"]


def translate_files(paths, procs, out_dir, extra=(), stem="ramref"):
    """Translate procs (names) of the modules in paths, plus every procedure
    of the modules in extra; writes <out_dir>/<stem>.c."""
    mods = {}
    for f in paths:
        mods.update(parse_modules(str(f)))
    want = [p.lower() for p in procs]
    for f in extra:
        mm = parse_modules(str(f))
        mods.update(mm)
        for m in mm.values():
            want += list(m.procs)
    tr = Translator(mods, want)
    bodies = tr.run()
    src = tr.emit(bodies)
    out = Path(out_dir)
    out.mkdir(parents=True, exist_ok=True)
    cpath = out / f"{stem}.c"
    cpath.write_text(src)
    return cpath, tr


def translate(ref_root, out_dir, extra=(), procs=None):
    """The kinetic-step routines of the reference tree at ref_root."""
    return translate_files([Path(ref_root) / f for f in REF_FILES], REF_PROCS if procs is None else procs,
                           out_dir, extra)


def compile_c(cpath, lib, check=False, cc=None):
    cc = cc or os.environ.get("CC", "gcc")
    cmd = [cc, "-O3", "-ffp-contract=off", "-fno-math-errno", "-fPIC", "-fopenmp", "-shared", "-std=gnu11",
           "-w", "-o", str(lib), str(cpath), "-lm"]
    if check:
        cmd.insert(1, "-DREF_CHECK")
    subprocess.run(cmd, check=True)
    return lib


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--ref", required=True, help="root of the reference's source tree")
    ap.add_argument("--out", required=True, help="output directory (oracle/_ref)")
    ap.add_argument("--extra", nargs="*", default=[], help="extra Fortran modules (driver)")
    ap.add_argument("--no-compile", action="store_true")
    a = ap.parse_args(argv)
    cpath, tr = translate(a.ref, a.out, a.extra)
    if not a.no_compile:
        compile_c(cpath, Path(a.out) / "libramref.so")
        compile_c(cpath, Path(a.out) / "libramref_check.so", check=True)
    print(cpath)


if __name__ == "__main__":
    main()
