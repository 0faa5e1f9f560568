"""Mechanical Julia-subset -> Python translator used ONLY to generate golden
fixtures from the reference's own source text (tests/golden/make_golden.py).

It handles exactly the constructs that appear in the reference's device
kernels and spectrum helpers: function definitions, if/elseif/else, for loops
over `range(a,b,step=s)` and `enumerate`, assignments to 1-based array
elements, broadcast operators on scalars, `x^n` with a literal integer n
(Julia's `literal_pow`, i.e. repeated multiplication), `÷`, `end` inside an
index, numeric-literal juxtaposition (`1j` == 1*j) and the handful of Base
functions the spectrum code calls.  Anything else raises, so a silent
mistranslation cannot slip into a fixture.

Evaluation order is Python's, which for + - * / chains is the same
left-to-right fold Julia uses for Float64 (n-ary `+`/`*` are `afoldl`).
"""
from __future__ import annotations

import math
import re

import numpy as np

_UNI = {"ϕ": "phi", "Γ": "Gam", "Σ": "Sig", "β": "beta", "γ": "gam",
        "θ": "theta", "ω": "omega", "ϵ": "eps", "÷": "//"}


# ---------------------------------------------------------------- runtime
class JArr:
    """1-based N-d array view with Julia indexing semantics."""

    def __init__(self, data: np.ndarray):
        self.d = data  # numpy, indexed in Julia order (i, j, k)

    def _conv(self, idx):
        if not isinstance(idx, tuple):
            idx = (idx,)
        out = []
        for ax, v in enumerate(idx):
            if isinstance(v, slice):
                if v.start is None and v.stop is None:
                    out.append(slice(None))
                else:
                    out.append(slice(v.start - 1, v.stop))
            elif isinstance(v, (list, np.ndarray)):
                out.append(np.asarray(v, dtype=np.int64) - 1)
            else:
                iv = int(v)
                if iv != v or iv < 1 or iv > self.d.shape[ax]:
                    raise IndexError(f"index {v} out of bounds for axis {ax} size {self.d.shape[ax]}")
                out.append(iv - 1)
        return tuple(out)

    def __getitem__(self, idx):
        r = self.d[self._conv(idx)]
        if isinstance(r, np.ndarray):
            return JArr(r.copy())
        return float(r)

    def __setitem__(self, idx, val):
        if isinstance(val, JArr):
            val = val.d
        self.d[self._conv(idx)] = val

    def __eq__(self, other):  # broadcast .== (only used with findall)
        return JArr(self.d == other)

    def __iter__(self):
        return (float(v) for v in self.d.ravel(order="F"))

    def size(self, dim):
        return self.d.shape[dim - 1]


def _size(A, dim=None):
    if isinstance(A, list):
        return len(A)
    if dim is None:
        return tuple(A.d.shape)
    return A.d.shape[dim - 1]


def _jrange(a, b, step=1):
    return range(int(a), int(b) + (1 if step > 0 else -1), int(step))


def _jenumerate(it):
    return ((i + 1, v) for i, v in enumerate(it))


def _push(lis, x):
    lis.append(x)
    return lis


def _sort(lis):
    if isinstance(lis, list):
        lis.sort()
        return lis
    raise TypeError("sort! on non-list")


def _unique(x):
    if isinstance(x, JArr):
        vals = x.d.ravel(order="F")
        seen, out = set(), []
        for v in vals:
            if float(v) not in seen:
                seen.add(float(v))
                out.append(float(v))
        return JArr(np.asarray(out))
    seen, out = set(), []
    for v in x:
        if v not in seen:
            seen.add(v)
            out.append(v)
    x[:] = out
    return x


def _zeros(shape, *rest):
    if rest:
        shape = (shape,) + rest
    if isinstance(shape, int):
        shape = (shape,)
    return JArr(np.zeros(shape))


def _sortslices(A, dims=1):
    if dims != 1:
        raise NotImplementedError
    d = A.d
    order = np.lexsort(tuple(d[:, c] for c in reversed(range(d.shape[1]))))
    return JArr(d[order].copy())


def _findall(mask):
    m = mask.d if isinstance(mask, JArr) else np.asarray(mask)
    return list(np.nonzero(m.ravel(order="F"))[0] + 1)


def _mean(x):
    v = x.d if isinstance(x, JArr) else np.asarray(x)
    return float(np.sum(v) / v.size)


def _jpow(x, n):
    if n == 2:
        return x * x
    if n == 3:
        return x * x * x
    raise NotImplementedError(f"literal_pow {n}")


RUNTIME = {
    "sqrt": math.sqrt, "sin": math.sin, "cos": math.cos, "exp": math.exp,
    "acos": math.acos, "asin": math.asin, "tan": math.tan, "abs": abs,
    "pi": math.pi, "size": _size, "jrange": _jrange, "jenumerate": _jenumerate,
    "push_b": _push, "sort_b": _sort, "unique_b": _unique, "zeros": _zeros,
    "sortslices": _sortslices, "findall": _findall, "mean": _mean,
    "_jpow": _jpow, "true": True, "false": False,
}


# ------------------------------------------------------------- translator
def _strip_comment(line: str) -> str:
    out, depth = [], 0
    for ch in line:
        if ch == "#":
            break
        out.append(ch)
    return "".join(out)


def _balance(s: str) -> int:
    return s.count("(") + s.count("[") - s.count(")") - s.count("]")


def extract_function(text: str, name: str, line_range: tuple[int, int] | None = None) -> list[str]:
    """Lines of the LAST definition of `name` inside `line_range` (1-based,
    inclusive; whole file when None).  Julia semantics: a later method
    definition with the same signature replaces the former."""
    lines = text.splitlines()
    if line_range is not None:
        lines = [l if line_range[0] <= n + 1 <= line_range[1] else "" for n, l in enumerate(lines)]
    pat = re.compile(r"^\s*(@views\s+)?function\s+" + re.escape(name) + r"\s*\(")
    starts = [i for i, l in enumerate(lines) if pat.match(l)]
    if not starts:
        raise KeyError(name)
    i0 = starts[-1]
    # join into statements, then follow block depth
    depth, out, buf = 0, [], ""
    i = i0
    while i < len(lines):
        raw = _strip_comment(lines[i])
        buf = (buf + " " + raw.strip()) if buf else raw.strip()
        i += 1
        if not buf:
            continue
        if _balance(buf) > 0 or re.search(r"[+\-*/=,(]\s*$", buf) and not buf.endswith("=="):
            continue
        stmt = buf
        buf = ""
        head = re.sub(r"^(@views|@inbounds)\s+", "", stmt)
        head = re.sub(r"^(@views|@inbounds)\s+", "", head)
        if re.match(r"^(function|if|for|while|begin)\b", head):
            depth += 1
        elif head == "end":
            depth -= 1
        out.append(stmt)
        if depth == 0:
            break
    return out


def _replace_end_in_index(s: str) -> str:
    """A[..., end-1, ...] -> A[..., size(A,p)-1, ...]."""
    res, i = [], 0
    while i < len(s):
        m = re.compile(r"([A-Za-z_]\w*)\[").match(s, i) if (i == 0 or not (s[i - 1].isalnum() or s[i - 1] == "_")) else None
        if m:
            name = m.group(1)
            j = m.end()
            depth, parts, cur = 1, [], []
            while depth:
                ch = s[j]
                if ch in "([":
                    depth += 1
                elif ch in ")]":
                    depth -= 1
                    if depth == 0:
                        break
                if ch == "," and depth == 1:
                    parts.append("".join(cur))
                    cur = []
                else:
                    cur.append(ch)
                j += 1
            parts.append("".join(cur))
            parts = [_replace_end_in_index(p) for p in parts]
            parts = [re.sub(r"\bend\b", f"size({name},{k + 1})", p) for k, p in enumerate(parts)]
            res.append(f"{name}[{','.join(parts)}]")
            i = j + 1
        else:
            res.append(s[i])
            i += 1
    return "".join(res)


def _left_operand_start(s: str, pos: int) -> int:
    j = pos - 1
    while j >= 0 and s[j] == " ":
        j -= 1
    while True:
        if s[j] in ")]":
            depth = 0
            while True:
                if s[j] in ")]":
                    depth += 1
                elif s[j] in "([":
                    depth -= 1
                    if depth == 0:
                        break
                j -= 1
            j -= 1
            # identifier directly before ( or [ belongs to the operand
            continue
        if s[j].isalnum() or s[j] in "_.":
            while j >= 0 and (s[j].isalnum() or s[j] in "_."):
                j -= 1
            if j >= 0 and s[j] in ")]":
                continue
            return j + 1
        return j + 1


def _translate_pow(s: str) -> str:
    while "^" in s:
        p = s.index("^")
        m = re.compile(r"\s*(\d+)").match(s, p + 1)
        if not m:
            raise NotImplementedError(f"non-literal exponent in: {s}")
        a = _left_operand_start(s, p)
        s = s[:a] + f"_jpow({s[a:p]},{m.group(1)})" + s[m.end():]
    return s


def translate_expr(s: str) -> str:
    s = s.replace(".==", "==")
    s = s.replace(".*", "*").replace(".+", "+").replace(".-", "-").replace("./", "/")
    s = re.sub(r"(?<![\w.])(\d+)([ijk])\b", r"\1*\2", s)   # 1j == 1*j
    s = re.sub(r"(\w)!(?!=)", r"\1_b", s)
    s = s.replace("&&", " and ").replace("||", " or ")
    s = _replace_end_in_index(s)
    s = _translate_pow(s)
    s = re.sub(r"\brange\(", "jrange(", s)
    s = re.sub(r"\benumerate\(", "jenumerate(", s)
    return s


def translate_function(lines: list[str], skip_thread_index: bool = True) -> str:
    py, ind = [], 0
    for stmt in lines:
        st = stmt
        for k, v in _UNI.items():
            st = st.replace(k, v)
        st = re.sub(r"\blambda\b", "lambda_", st)
        st = re.sub(r"^(@views|@inbounds)\s+", "", st.strip())
        st = re.sub(r"^(@views|@inbounds)\s+", "", st)
        st = st.replace("@views ", "").replace("@inbounds ", "")
        if st.startswith("function"):
            m = re.match(r"function\s+([\w!]+)\((.*)\)$", st)
            name = m.group(1).replace("!", "_b")
            args = m.group(2)
            if ";" in args:
                a, kw = args.split(";", 1)
                args = a + ", *, " + kw.replace("false", "False").replace("true", "True")
            extra = ", i, j, k" if skip_thread_index and "blockIdx" in " ".join(lines) else ""
            py.append("    " * ind + f"def {name}({args}{extra}):")
            ind += 1
            continue
        if "blockIdx()" in st:
            continue
        if st.startswith("println") or st.startswith("@cuprintln"):
            continue
        if st == "end":
            ind -= 1
            continue
        if st.startswith("elseif"):
            py.append("    " * (ind - 1) + "elif " + translate_expr(st[6:].strip()) + ":")
            continue
        if st == "else":
            py.append("    " * (ind - 1) + "else:")
            continue
        if st.startswith("if "):
            py.append("    " * ind + "if " + translate_expr(st[3:].strip()) + ":")
            ind += 1
            continue
        if st.startswith("for "):
            py.append("    " * ind + "for " + translate_expr(st[4:].strip()) + ":")
            ind += 1
            continue
        if st == "return":
            py.append("    " * ind + "return None")
            continue
        py.append("    " * ind + translate_expr(st))
    return "\n".join(py) + "\n"


def load_functions(path: str, names: list[str], namespace: dict | None = None,
                   line_range: tuple[int, int] | None = None) -> dict:
    text = open(path, encoding="utf-8").read()
    ns = dict(RUNTIME) if namespace is None else namespace
    for n in names:
        src = translate_function(extract_function(text, n, line_range))
        exec(compile(src, f"<{n}>", "exec"), ns)
    return ns


def signature(path: str, name: str) -> list[str]:
    text = open(path, encoding="utf-8").read()
    first = extract_function(text, name)[0]
    for k, v in _UNI.items():
        first = first.replace(k, v)
    first = re.sub(r"\blambda\b", "lambda_", first)
    m = re.search(r"\((.*)\)\s*$", first)
    return [a.strip() for a in m.group(1).split(";")[0].split(",") if a.strip()]
