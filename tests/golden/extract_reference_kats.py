"""Extract the known-answer tables of ImageFiltering.jl's own test suite into
``reference_kats.json``.

The reference is Julia and cannot run here, so its golden tables are read as
text from its test files and parsed with a small Julia-literal reader.  The
JSON this writes is committed; this script is the record of how it was made
and needs the reference source tree, whose path is its one command-line
argument.  Tests never read the reference tree.

Tables extracted (paths relative to the reference tree):
  * test/border.jl   -- every ``padarray(A, <border>) == OffsetArray([...], offs)``
                        and ``== [...]`` table, with the ``A`` in scope
                        (5x5 goldens 67-86 etc., arrays smaller than the pad,
                        asymmetric lo/hi)
  * test/mapwindow.jl -- the 1-D ``mapwindow(extrema, A, w)`` tables (even and
                        odd windows, Lemire path), the 1-D median tables and the
                        4x5 (3,3) median table
  * test/nd.jl       -- the cascade-trimming tables A1/A2 and the (k1,) /
                        copy-kernel results on 1:8
"""
import json
import os
import re
import sys

if len(sys.argv) != 2:
    sys.exit("usage: extract_reference_kats.py <ImageFiltering.jl source tree>")
REF = sys.argv[1]
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_kats.json")


# ----------------------------------------------------------------------------
# A small reader for the Julia literals that appear in those tables
# ----------------------------------------------------------------------------
def _num(tok):
    tok = tok.strip()
    if re.fullmatch(r"[-+]?\d+", tok):
        return int(tok)
    return float(tok)


def _split_top(s, sep):
    """Split on `sep` at bracket depth 0."""
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch in "([":
            depth += 1
        elif ch in ")]":
            depth -= 1
        if ch == sep and depth == 0:
            out.append(cur)
            cur = ""
        else:
            cur += ch
    out.append(cur)
    return out


def parse_elem(s):
    s = s.strip()
    if s.startswith("(") and s.endswith(")"):
        return [parse_elem(x) for x in _split_top(s[1:-1], ",")]
    if s.startswith('"') and s.endswith('"'):
        return s[1:-1]
    return _num(s)


def parse_array(s):
    """Parse `[...]`: comma vector, or matrix with spaces and ; / newlines.
    Matrices come back as a list of rows."""
    s = s.strip()
    assert s[0] == "[" and s[-1] == "]", s
    body = s[1:-1].strip()
    rows = [r for r in re.split(r";|\n", body) if r.strip()]
    if len(rows) == 1 and len(_split_top(rows[0], ",")) > 1:
        return [parse_elem(x) for x in _split_top(rows[0], ",") if x.strip()]
    mat = []
    for r in rows:
        toks = r.split()
        mat.append([parse_elem(t) for t in toks])
    if len(mat) == 1:
        return {"row": mat[0]}
    return mat


def take_bracket(text, i):
    """Return the substring starting at text[i]=='[' up to its matching ']'."""
    assert text[i] == "["
    depth = 0
    for j in range(i, len(text)):
        if text[j] == "[":
            depth += 1
        elif text[j] == "]":
            depth -= 1
            if depth == 0:
                return text[i:j + 1], j + 1
    raise ValueError("unbalanced")


def parse_border(spec):
    """Pad(:style,(lo..),(hi..)) / Pad(:style,(lo..),()) / Pad(1,1) / Fill(v,(lo),(hi))."""
    spec = spec.strip()
    m = re.fullmatch(r"Fill\(\s*(-?\d+)\s*,\s*\(([^)]*)\)\s*,\s*\(([^)]*)\)\s*\)", spec)
    if m:
        return {"style": "fill", "fill": int(m.group(1)),
                "lo": [int(x) for x in m.group(2).split(",") if x.strip()],
                "hi": [int(x) for x in m.group(3).split(",") if x.strip()]}
    m = re.fullmatch(r"Pad\(\s*:(\w+)\s*,\s*\(([^)]*)\)\s*,\s*\(([^)]*)\)\s*\)", spec)
    if m:
        lo = [int(x) for x in m.group(2).split(",") if x.strip()]
        hi = [int(x) for x in m.group(3).split(",") if x.strip()]
        n = max(len(lo), len(hi))
        lo = lo or [0] * n
        hi = hi or [0] * n
        return {"style": m.group(1), "lo": lo, "hi": hi}
    m = re.fullmatch(r"Pad\(\s*(\d+)\s*,\s*(\d+)\s*\)", spec)
    if m:   # Pad(m, n) == Pad(:replicate, (m,n), (m,n))
        v = [int(m.group(1)), int(m.group(2))]
        return {"style": "replicate", "lo": v, "hi": v}
    return None


def eval_A(expr):
    """Values of the `A = ...` / `Ao = ...` assignments in test/border.jl."""
    expr = expr.strip()
    m = re.fullmatch(r"reshape\(1:(\d+),\s*(\d+),\s*(\d+)\)", expr)
    if m:
        n, r, c = int(m.group(1)), int(m.group(2)), int(m.group(3))
        vals = list(range(1, n + 1))
        return [[vals[i + r * j] for j in range(c)] for i in range(r)]
    m = re.fullmatch(r"OffsetArray\(reshape\(1:(\d+),\s*(\d+),\s*(\d+)\),\s*-1,\s*-1\)", expr)
    if m:
        return eval_A("reshape(1:%s, %s, %s)" % m.groups())
    if expr.startswith("["):
        v = parse_array(expr)
        if isinstance(v, list) and v and isinstance(v[0], list) and all(isinstance(x, (int, float)) for x in v[0]):
            return v
    return None


def border_kats():
    path = os.path.join(REF, "test", "border.jl")
    text = open(path).read()
    kats = []
    scope = {}
    pat_assign = re.compile(r"^\s*(A|Ao)\s*=\s*(.+)$", re.M)
    pat_test = re.compile(r"padarray\((A|Ao),\s*((?:Pad|Fill)\((?:[^()]|\([^()]*\))*\))\)\)\s*==\s*")
    events = []
    for m in pat_assign.finditer(text):
        events.append((m.start(), "assign", m))
    for m in pat_test.finditer(text):
        events.append((m.start(), "test", m))
    events.sort(key=lambda e: e[0])
    for start, kind, m in events:
        if kind == "assign":
            val = eval_A(m.group(2))
            scope[m.group(1)] = val
            continue
        name, spec = m.group(1), m.group(2)
        b = parse_border(spec)
        if b is None or scope.get(name) is None:
            continue
        j = m.end()
        line = text.count("\n", 0, start) + 1
        if text.startswith("OffsetArray(", j):
            j2 = j + len("OffsetArray(")
            while text[j2].isspace():
                j2 += 1
            arr, k = take_bracket(text, j2)
            offs = re.match(r"\s*,\s*\(([^)]*)\)\)", text[k:])
            expected = parse_array(arr)
            offsets = [int(x) for x in offs.group(1).split(",")]
        elif text[j] == "[":
            arr, k = take_bracket(text, j)
            expected = parse_array(arr)
            offsets = [0, 0]
        else:
            continue
        if isinstance(expected, dict):
            expected = [expected["row"]]
        kats.append({"source": "test/border.jl:%d" % line, "A": scope[name], "border": b,
                     "expected": expected, "offsets": offsets,
                     "array_first_index": 0 if name == "Ao" else 1})
    return kats


def mapwindow_kats():
    path = os.path.join(REF, "test", "mapwindow.jl")
    lines = open(path).read().split("\n")
    ext, med = [], []
    A = None
    for i, ln in enumerate(lines):
        m = re.match(r"\s*A = (\[[-0-9., ]+\])\s*$", ln)
        if m:
            A = parse_array(m.group(1))
        m = re.match(r"\s*mm = mapwindow\(extrema, A, (\d+)\)", ln)
        if m and A is not None and i + 1 < len(lines):
            t = re.match(r"\s*@test mm == (\[.*\])\s*$", lines[i + 1])
            if t:
                if t.group(1) == "[(a,a) for a in A]":   # identity window
                    exp = [[a, a] for a in A]
                else:
                    exp = parse_array(t.group(1))
                ext.append({"source": "test/mapwindow.jl:%d" % (i + 2), "A": A,
                            "window": int(m.group(1)), "expected": exp})
    text = "\n".join(lines)
    # 1-D medians on a and b
    vals = {}
    for m in re.finditer(r"^\s*(a|b) = (\[[-0-9, ]+\])", text, re.M):
        vals[m.group(1)] = parse_array(m.group(2))
    for m in re.finditer(r"@test mapwindow\(f, (a|b), (-?\d+):(-?\d+)\) == (a|\[[-0-9, ]+\])", text):
        exp = vals["a"] if m.group(4) == "a" else parse_array(m.group(4))
        line = text.count("\n", 0, m.start()) + 1
        med.append({"source": "test/mapwindow.jl:%d" % line, "A": vals[m.group(1)],
                    "window_first": [int(m.group(2))],
                    "window_len": [int(m.group(3)) - int(m.group(2)) + 1], "expected": exp})
    # the 4x5 (3,3) table
    m = re.search(r"A = (\[1 5 -2 3 7;.*?\])\s*\n\s*@test mapwindow\(f, A, \(3,3\)\) == (\[.*?\])", text, re.S)
    if m:
        line = text.count("\n", 0, m.start()) + 1
        med.append({"source": "test/mapwindow.jl:%d" % line, "A": parse_array(m.group(1)),
                    "window_first": [-1, -1], "window_len": [3, 3],
                    "expected": parse_array(m.group(2))})
    return ext, med


def nd_kats():
    path = os.path.join(REF, "test", "nd.jl")
    text = open(path).read()
    out = []
    for name in ("A1", "A2"):
        m = re.search(r"@test %s ≈ OffsetArray\((\[[-0-9., ]+\]),\s*(-?\d+):(-?\d+)\)" % name, text)
        line = text.count("\n", 0, m.start()) + 1
        out.append({"source": "test/nd.jl:%d" % line, "name": name,
                    "expected": parse_array(m.group(1)), "first": int(m.group(2))})
    m = re.search(r"@test imfilter\(img, \(k1,\)\) ≈ (\[[-0-9., ]+\])", text)
    line = text.count("\n", 0, m.start()) + 1
    out.append({"source": "test/nd.jl:%d" % line, "name": "k1_on_1to8",
                "expected": parse_array(m.group(1))})
    return out


def main():
    ext, med = mapwindow_kats()
    kats = {
        "reference": "ImageFiltering.jl v0.7.12 test suite",
        "padarray": border_kats(),
        "extrema_lemire_1d": ext,
        "median": med,
        "cascade_1d": nd_kats(),
    }
    with open(OUT, "w") as f:
        json.dump(kats, f, indent=1)
    print("wrote", OUT, {k: len(v) for k, v in kats.items() if isinstance(v, list)})


if __name__ == "__main__":
    main()
