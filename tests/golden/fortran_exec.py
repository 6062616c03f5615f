"""Execute a subset of Fortran 90 source statements in Python, literally.

Used only to generate golden fixtures from the MGLC reference's own source
files (no Fortran compiler is available in this environment).  Each reference
subroutine is translated statement by statement into Python and run on small
grids; Python floats are IEEE binary64 with round-to-nearest and no FMA, and
binary operators of equal precedence evaluate left to right, as in Fortran, so
the results follow the source's arithmetic exactly.

Supported subset (all the hot-path subroutines need): module parameters and
declarations, ``allocate``, ``data``, array constructors with implied do,
``do``/``do while``/``if``/``elseif``/``else``, assignments to scalars, array
elements and whole arrays, intrinsic calls, cpp ``#ifdef``/``#ifndef``/
``#else``/``#endif``/``#define``.  MPI calls are run as on a single rank
(``MPI_Allreduce`` copies, everything else is a no-op); I/O is skipped.
Default-real literals (``1e-6``, ``2.0``) are rounded to binary32 first.
"""
from __future__ import annotations

import math
import re

import numpy as np


class FArr:
    """Fortran array with explicit lower bounds (column-major semantics)."""

    def __init__(self, bounds, dtype=np.float64, fill=np.nan):
        self.lb = tuple(b[0] for b in bounds)
        shape = tuple(b[1] - b[0] + 1 for b in bounds)
        if dtype == np.int64 and isinstance(fill, float) and math.isnan(fill):
            fill = -999999
        # store reversed so that the first index is fastest, like Fortran
        self.a = np.full(shape[::-1], fill, dtype=dtype)
        self.rank = len(bounds)

    def _key(self, idx):
        if not isinstance(idx, tuple):
            idx = (idx,)
        return tuple(int(i) - l for i, l in zip(idx, self.lb))[::-1]

    def __getitem__(self, idx):
        v = self.a[self._key(idx)]
        return float(v) if self.a.dtype == np.float64 else int(v)

    def __setitem__(self, idx, val):
        self.a[self._key(idx)] = val

    def fill(self, val):
        if isinstance(val, FArr):
            self.a[...] = val.a
        else:
            self.a[...] = val

    def numpy(self):
        return self.a.copy()


def _r4(x):
    return float(np.float32(x))


def _fmod(a, b):
    if isinstance(a, int) and isinstance(b, int):
        return int(math.fmod(a, b))
    return math.fmod(a, b)


def _fint(x):
    return int(x)  # truncation toward zero


def _sq(x):
    return x * x


def _nint(x):
    return int(math.floor(x + 0.5)) if x >= 0 else -int(math.floor(-x + 0.5))


INTRINSICS = {
    "dsqrt": "math.sqrt", "sqrt": "math.sqrt", "dabs": "abs", "abs": "abs", "dble": "float",
    "real": "float", "int": "_fint", "nint": "_nint", "mod": "_fmod", "atan": "math.atan",
    "datan": "math.atan", "dexp": "math.exp", "exp": "math.exp", "max": "max", "min": "min",
    "dmax1": "max", "dmin1": "min", "floor": "math.floor", "dcos": "math.cos",
    "cos": "math.cos", "dsin": "math.sin", "sin": "math.sin", "sign": "math.copysign",
}

REL = [(r"\.eq\.", " == "), (r"\.ne\.", " != "), (r"\.lt\.", " < "), (r"\.le\.", " <= "),
       (r"\.gt\.", " > "), (r"\.ge\.", " >= "), (r"\.and\.", " and "), (r"\.or\.", " or "),
       (r"\.not\.", " not "), (r"\.true\.", " True "), (r"\.false\.", " False "),
       (r"/=", " != ")]

NUM = re.compile(r"(?<![\w.])(\d+\.\d*|\.\d+|\d+)([de][+-]?\d+)?(_\d+)?(?![\w])", re.I)


def preprocess(text: str, defines: set[str], undefines=frozenset()) -> list[str]:
    """cpp subset, comment stripping and continuation joining.

    ``undefines`` lists macros whose ``#define`` lines in the source are ignored,
    so that a caller can select another boundary-condition variant."""
    out, stack = [], []
    active = True
    for raw in text.splitlines():
        s = raw.strip()
        if s.startswith("#"):
            toks = s[1:].split()
            d = toks[0] if toks else ""
            if d == "define":
                if active and toks[1] not in undefines:
                    defines.add(toks[1])
            elif d == "ifdef":
                stack.append(active)
                active = active and toks[1] in defines
            elif d == "ifndef":
                stack.append(active)
                active = active and toks[1] not in defines
            elif d == "else":
                active = stack[-1] and not active
            elif d == "endif":
                active = stack.pop()
            continue
        if active:
            out.append(raw)
    # strip comments (no '!' inside strings matters: I/O lines are dropped later)
    lines = []
    for l in out:
        in_str, q, res = False, "", []
        for ch in l:
            if in_str:
                res.append(ch)
                if ch == q:
                    in_str = False
            elif ch in "'\"":
                in_str, q = True, ch
                res.append(ch)
            elif ch == "!":
                break
            else:
                res.append(ch)
        lines.append("".join(res).rstrip())
    joined, buf = [], ""
    for l in lines:
        t = l.strip()
        if not t and not buf:
            continue
        if buf and t.startswith("&"):
            t = t[1:]
        if t.endswith("&"):
            buf += t[:-1] + " "
            continue
        buf += t
        if buf.strip():
            joined.append(buf.strip())
        buf = ""
    return joined


def split_top(s: str, sep=","):
    parts, depth, cur = [], 0, []
    for ch in s:
        if ch in "([":
            depth += 1
        elif ch in ")]":
            depth -= 1
        if ch == sep and depth == 0:
            parts.append("".join(cur))
            cur = []
        else:
            cur.append(ch)
    parts.append("".join(cur))
    return [p.strip() for p in parts]


class Program:
    def __init__(self, defines=None):
        self.ns = {"math": math, "np": np, "FArr": FArr, "_r4": _r4, "_fmod": _fmod,
                   "_fint": _fint, "_nint": _nint, "_sq": _sq}
        self.random_values: list[float] = []  # values returned by random_number, in order
        self.ns["_rand"] = lambda: float(self.random_values.pop(0))
        self.sub_args: dict[str, list[str]] = {}
        self.defines = set(defines or ())
        self.arrays: set[str] = set()
        self.int_arrays: set[str] = set()
        self.scalars: set[str] = set()
        self.subs: dict[str, list[str]] = {}
        self.overrides: dict[str, object] = {}

    # ---------------- expression translation ----------------
    @staticmethod
    def _squares(e: str) -> str:
        """Rewrite OPERAND**2.0d0 (or **2) as _sq(OPERAND): the square as a product."""
        pat = re.compile(r"\*\*\s*2(\.0*)?(d0)?(?![\w.])", re.I)
        while True:
            m = pat.search(e)
            if not m:
                return e
            k = m.start() - 1
            while k >= 0 and e[k] == " ":
                k -= 1
            end = k + 1
            if e[k] == ")":
                depth = 0
                while k >= 0:
                    if e[k] == ")":
                        depth += 1
                    elif e[k] == "(":
                        depth -= 1
                        if depth == 0:
                            break
                    k -= 1
                k -= 1
                while k >= 0 and (e[k].isalnum() or e[k] == "_"):
                    k -= 1
            else:
                while k >= 0 and (e[k].isalnum() or e[k] in "_."):
                    k -= 1
            start = k + 1
            e = e[:start] + "_sq(" + e[start:end] + ")" + e[m.end():]

    def expr(self, e: str, local_arrays=frozenset()) -> str:
        e = self._squares(e.strip())
        # array constructor (/ ... /)
        if e.startswith("(/") and e.endswith("/)"):
            return self._constructor(e[2:-2], local_arrays)
        # protect string literals
        strings = []

        def _s(m):
            strings.append(m.group(0))
            return f"__S{len(strings) - 1}__"

        e = re.sub(r"'[^']*'|\"[^\"]*\"", _s, e)
        for pat, rep in REL:
            e = re.sub(pat, rep, e, flags=re.I)

        def num(m):
            mant, ex, kind = m.group(1), m.group(2), m.group(3)
            if ex is None and "." not in mant:
                return mant if kind is None else mant  # integer literal
            if ex is not None and ex[0] in "dD":
                return f"{mant}e{ex[1:]}" if mant.replace('.', '') else mant
            if kind == "_8":
                return mant + (("e" + ex[1:]) if ex else "")
            val = mant + (("e" + ex[1:]) if ex else "")
            return f"_r4({val})"

        e = NUM.sub(num, e)

        # names followed by '(' : array refs or intrinsic/function calls
        def name(m):
            n = m.group(1)
            nl = n.lower()
            if nl in ("and", "or", "not", "true", "false") or nl.startswith("__s"):
                return n
            return nl

        e = re.sub(r"(?<![\w.])([A-Za-z_]\w*)", name, e)
        out, i = [], 0
        while i < len(e):
            m = re.match(r"([a-z_]\w*)\s*\(", e[i:])
            if m and (i == 0 or not (e[i - 1].isalnum() or e[i - 1] == "_")):
                n = m.group(1)
                if n in ("and", "or", "not", "_r4", "_sq", "_rand"):
                    out.append(e[i:i + m.end()])
                    i += m.end()
                    continue
                j = i + m.end()
                depth, k = 1, j
                while depth:
                    if e[k] == "(":
                        depth += 1
                    elif e[k] == ")":
                        depth -= 1
                    k += 1
                inner = e[j:k - 1]
                args = [self.expr(a, local_arrays) for a in split_top(inner)]
                if n in self.arrays or n in local_arrays:
                    out.append(f"{n}[{', '.join(args)}]")
                elif n in INTRINSICS:
                    out.append(f"{INTRINSICS[n]}({', '.join(args)})")
                else:
                    raise ValueError(f"unknown function or array '{n}' in: {e}")
                i = k
            else:
                out.append(e[i])
                i += 1
        e = "".join(out)
        for idx, s in enumerate(strings):
            e = e.replace(f"__S{idx}__", s)
        return e

    def _constructor(self, body, local_arrays):
        items = []
        for it in split_top(body):
            m = re.match(r"^\((.*),\s*(\w+)\s*=\s*(.*),\s*(.*)\)$", it)
            if m:
                val, var, lo, hi = m.groups()
                items.append(f"*[{self.expr(val, local_arrays)} for {var.lower()} in range({self.expr(lo)}, {self.expr(hi)}+1)]")
            else:
                items.append(self.expr(it, local_arrays))
        return "[" + ", ".join(items) + "]"

    # ---------------- module parsing ----------------
    def load_module(self, lines: list[str]):
        in_mod = False
        for st in lines:
            sl = st.lower()
            if re.match(r"^module\s+\w+", sl):
                in_mod = True
                continue
            if re.match(r"^end\s*module", sl):
                in_mod = False
                continue
            if not in_mod:
                continue
            if sl.startswith("implicit") or sl.startswith("use "):
                continue
            if sl.startswith("data "):
                self._data(st)
                continue
            if "::" in st:
                self._decl(st, module=True)

    def _data(self, st):
        for m in re.finditer(r"(\w+)\s*/([^/]*)/", st[5:]):
            n = m.group(1).lower()
            vals = [self.expr(v) for v in split_top(m.group(2))]
            arr = self.ns[n]
            for idx, v in enumerate(vals):
                arr[arr.lb[0] + idx] = eval(v, self.ns)

    def _bounds(self, dims: str, local_env=None):
        bs = []
        for d in split_top(dims):
            if d.strip() == ":":
                return None
            if ":" in d:
                lo, hi = d.split(":")
            else:
                lo, hi = "1", d
            env = dict(self.ns)
            if local_env:
                env.update(local_env)
            bs.append((int(eval(self.expr(lo), env)), int(eval(self.expr(hi), env))))
        return bs

    def _decl(self, st, module=False, local_arrays=None, code=None, indent=""):
        head, rest = st.split("::", 1)
        hl = head.lower()
        is_int = hl.strip().startswith("integer")
        is_param = "parameter" in hl
        if hl.strip().startswith("character"):
            return
        for item in split_top(rest):
            m = re.match(r"^(\w+)\s*(\(([^=]*)\))?\s*(=\s*(.*))?$", item.strip(), re.S)
            if not m:
                raise ValueError(item)
            n = m.group(1).lower()
            dims = m.group(3)
            init = m.group(5)
            if module:
                if n in self.overrides:
                    self.ns[n] = self.overrides[n]
                    if dims:
                        self.arrays.add(n)
                    else:
                        self.scalars.add(n)
                    continue
                if dims:
                    self.arrays.add(n)
                    if is_int:
                        self.int_arrays.add(n)
                    bs = self._bounds(dims)
                    if bs is not None:
                        arr = FArr(bs, np.int64 if is_int else np.float64)
                        if init:
                            vals = eval(self.expr(init), self.ns)
                            arr.a[...] = np.array(vals).reshape(arr.a.shape[::-1]).T
                        self.ns[n] = arr
                else:
                    self.scalars.add(n)
                    if init is not None:
                        v = eval(self.expr(init), self.ns)
                        self.ns[n] = (int(v) if is_int else float(v)) if not isinstance(v, bool) else v
                    elif n not in self.ns:
                        self.ns[n] = 0 if is_int else float("nan")
            else:
                if dims and dims.replace(",", "").replace(":", "").strip() == "":
                    local_arrays.add(n)  # deferred shape: created by allocate
                elif dims:
                    local_arrays.add(n)
                    code.append(f"{indent}{n} = FArr({self._bounds_src(dims)}, "
                                f"{'np.int64' if is_int else 'np.float64'})")
                    if init:
                        code.append(f"{indent}{n}.fill({self.expr(init)})")
                else:
                    self._local_scalars.add(n)
                    if init is not None:
                        code.append(f"{indent}{n} = {self.expr(init)}")
                    elif n not in getattr(self, "_dummies", []):
                        # Fortran leaves locals undefined; bind them so that they can be
                        # passed as output arguments (NaN exposes any read before write)
                        code.append(f"{indent}{n} = {'0' if is_int else 'float(\'nan\')'}")

    def _bounds_src(self, dims):
        out = []
        for d in split_top(dims):
            lo, hi = d.split(":") if ":" in d else ("1", d)
            out.append(f"({self.expr(lo)}, {self.expr(hi)})")
        return "[" + ", ".join(out) + "]"

    # ---------------- subroutines ----------------
    def load_subroutines(self, lines: list[str]):
        cur, body = None, []
        for st in lines:
            sl = st.lower()
            m = re.match(r"^subroutine\s+(\w+)\s*(\((.*)\))?", sl)
            if m and cur is None:
                cur, body = m.group(1), []
                self.sub_args[cur] = [a.strip() for a in m.group(3).split(",")] if m.group(3) and m.group(3).strip() else []
                continue
            if cur and re.match(r"^end\s*subroutine", sl):
                self.subs[cur] = body
                cur = None
                continue
            if cur:
                body.append(st)

    def compile(self, name: str):
        body = self.subs[name]
        self._dummies = self.sub_args.get(name, [])
        local_arrays: set[str] = set()
        self._local_scalars: set[str] = set()
        code: list[str] = []
        ind = "    "
        assigned = set()
        for st in body:
            sl = st.lower().strip()
            if sl.startswith(("use ", "implicit")) or sl == "use":
                continue
            if re.match(r"^\d+\s+format", sl):
                continue
            if "::" in st and re.match(r"^(real|integer|logical|character|double)", sl):
                self._decl(st, local_arrays=local_arrays, code=code, indent=ind)
                continue
            if re.match(r"^(write|print|open|close|read)\b", sl):
                code.append(f"{ind}pass")
                continue
            if sl == "return":
                code.append(f"{ind}return {self._ret()}")
                continue
            if sl == "stop" or sl.startswith("stop "):
                code.append(f"{ind}raise RuntimeError('reference STOP')")
                continue
            m = re.match(r"^do\s+while\s*\((.*)\)$", sl)
            if m:
                code.append(f"{ind}while {self.expr(st[st.lower().index('(') + 1:st.rindex(')')], local_arrays)}:")
                ind += "    "
                continue
            m = re.match(r"^do\s+(\w+)\s*=\s*(.*)$", st, re.I)
            if m:
                v = m.group(1).lower()
                parts = split_top(m.group(2))
                step = self.expr(parts[2], local_arrays) if len(parts) > 2 else "1"
                lo, hi = self.expr(parts[0], local_arrays), self.expr(parts[1], local_arrays)
                stop = f"({hi})+1" if step == "1" else f"({hi})+(1 if ({step})>0 else -1)"
                code.append(f"{ind}for {v} in range({lo}, {stop}, {step}):")
                ind += "    "
                continue
            if re.match(r"^end\s*do$", sl):
                ind = ind[:-4]
                continue
            m = re.match(r"^(else\s*if)\s*\((.*)\)\s*then$", st, re.I)
            if m:
                ind = ind[:-4]
                code.append(f"{ind}elif {self.expr(m.group(2), local_arrays)}:")
                ind += "    "
                continue
            if sl == "else":
                ind = ind[:-4]
                code.append(f"{ind}else:")
                ind += "    "
                continue
            if re.match(r"^end\s*if$", sl):
                ind = ind[:-4]
                continue
            m = re.match(r"^if\s*\((.*)\)\s*then$", st, re.I)
            if m:
                code.append(f"{ind}if {self.expr(m.group(1), local_arrays)}:")
                ind += "    "
                continue
            m = re.match(r"^if\s*(\(.*)$", st, re.I)
            if m:  # single-line if
                cond, rest = self._split_cond(m.group(1))
                code.append(f"{ind}if {self.expr(cond, local_arrays)}:")
                code.extend(self._simple(rest, ind + "    ", local_arrays, assigned))
                continue
            if re.match(r"^allocate\s*\(", sl):
                inner = st[st.index("(") + 1:st.rindex(")")]
                for item in split_top(inner):
                    mm = re.match(r"^(\w+)\s*\((.*)\)$", item.strip())
                    n = mm.group(1).lower()
                    dt = "np.int64" if n in self.int_arrays else "np.float64"
                    code.append(f"{ind}globals()['{n}'] = FArr({self._bounds_src(mm.group(2))}, {dt})")
                continue
            if re.match(r"^deallocate\s*\(", sl):
                continue
            code.extend(self._simple(st, ind, local_arrays, assigned))
        glob = sorted((assigned & self.scalars) - self._local_scalars - set(self._dummies))
        src = [f"def {name}({', '.join(self._dummies)}):"]
        if glob:
            src.append("    global " + ", ".join(glob))
        src.append("    pass")
        src.extend(code)
        src.append(f"    return {self._ret()}")
        return "\n".join(src)

    def _ret(self):
        return "(" + "".join(d + ", " for d in self._dummies) + ")" if self._dummies else "None"

    def _split_cond(self, s):
        depth = 0
        for k, ch in enumerate(s):
            if ch == "(":
                depth += 1
            elif ch == ")":
                depth -= 1
                if depth == 0:
                    return s[1:k], s[k + 1:].strip()
        raise ValueError(s)

    def _simple(self, st, ind, local_arrays, assigned):
        sl = st.lower().strip()
        if sl.startswith("call "):
            m = re.match(r"^call\s+(\w+)\s*(\((.*)\))?$", st.strip(), re.I)
            n = m.group(1).lower()
            args = split_top(m.group(3)) if m.group(3) else []
            if n == "random_number":
                tgt = args[0].strip().lower()
                return [f"{ind}{self.expr(args[0], local_arrays) if '(' in tgt else tgt} = _rand()"]
            if n == "random_seed":
                outs = [a.split("=")[1].strip().lower() for a in args if a.lower().startswith("size")]
                return [f"{ind}{o} = 1" for o in outs] or [f"{ind}pass"]
            if n == "mpi_abort":
                return [f"{ind}raise RuntimeError('reference MPI_Abort')"]
            if n == "mpi_allreduce":
                src, dst = self.expr(args[0], local_arrays), args[1].strip().lower()
                assigned.add(dst)
                if dst in self.arrays:
                    return [f"{ind}{dst}.fill({src})"]
                return [f"{ind}{dst} = {src}"]
            if n.startswith("mpi_") or n.startswith("omp_"):
                return [f"{ind}pass"]
            if n in self.subs:
                if not args:
                    return [f"{ind}{n}()"]
                # by-reference: plain names and array elements receive the dummies' final values
                out = [f"{ind}_r = {n}({', '.join(self.expr(a, local_arrays) for a in args)})"]
                for k, a in enumerate(args):
                    a = a.strip()
                    mm = re.match(r"^(\w+)\s*(\((.*)\))?$", a)
                    if not mm:
                        continue
                    nm = mm.group(1).lower()
                    if nm in INTRINSICS and nm not in self.arrays and nm not in local_arrays:
                        continue
                    if mm.group(2):
                        if nm in self.arrays or nm in local_arrays:
                            out.append(f"{ind}{self.expr(a, local_arrays)} = _r[{k}]")
                    elif not re.match(r"^\d", nm):
                        out.append(f"{ind}{nm} = _r[{k}]")
                        assigned.add(nm)
                return out
            return [f"{ind}pass  # skipped call {n}"]
        if re.match(r"^(write|print)\b", sl):
            return [f"{ind}pass"]
        if sl == "exit":
            return [f"{ind}break"]
        if sl == "stop" or sl.startswith("stop "):
            return [f"{ind}raise RuntimeError('reference STOP')"]
        # assignment
        depth, eq = 0, -1
        for k, ch in enumerate(st):
            if ch == "(":
                depth += 1
            elif ch == ")":
                depth -= 1
            elif ch == "=" and depth == 0 and st[k + 1:k + 2] != "=" and st[k - 1:k] not in "<>/=":
                eq = k
                break
        if eq < 0:
            raise ValueError("cannot translate statement: " + st)
        lhs, rhs = st[:eq].strip(), st[eq + 1:].strip()
        rhs_py = self.expr(rhs, local_arrays)
        m = re.match(r"^(\w+)\s*(\((.*)\))?$", lhs)
        n = m.group(1).lower()
        if m.group(2):
            idx = [self.expr(a, local_arrays) for a in split_top(m.group(3))]
            return [f"{ind}{n}[{', '.join(idx)}] = {rhs_py}"]
        if n in self.arrays or n in local_arrays:
            return [f"{ind}{n}.fill({rhs_py})"]
        assigned.add(n)
        return [f"{ind}{n} = {rhs_py}"]

    def build(self, names):
        for n in names:
            src = self.compile(n)
            exec(compile(src, f"<fortran:{n}>", "exec"), self.ns)

    def call(self, name):
        self.ns[name]()
