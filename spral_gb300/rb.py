"""Rutherford-Boeing matrix files (the format of src/rutherford_boeing.f90),
assembled matrices: read and write.

Header (four 80-column lines): title (72) + identifier (8); card counts;
type code (real/integer/pattern, symmetric/unsymmetric/..., assembled) with
m, n, nnz and a zero; the Fortran formats of the pointer, index and value
sections.  The data follow in those fixed-width formats, 1-based.
Symmetric matrices store their lower triangle by columns.
"""
import re

import numpy as np

_FMT = re.compile(r"\(\s*(?:\d+\s*P\s*,?\s*)?(\d*)\s*([IEDFGiedfg])\s*(\d+)")


def _parse_format(fmt):
    """(count per line, field width) of a Fortran format such as (10I8),
    (1P,4E20.12) or (3D26.16)."""
    m = _FMT.search(fmt)
    if not m:
        raise ValueError(f"unsupported Fortran format {fmt!r}")
    per = int(m.group(1)) if m.group(1) else 1
    return per, int(m.group(3))


def _read_fields(lines, start, count, fmt, conv):
    per, width = _parse_format(fmt)
    out, ln = [], start
    while len(out) < count:
        if ln >= len(lines):
            raise ValueError("file ends before all entries were read")
        s = lines[ln].rstrip("\n")
        for k in range(per):
            if len(out) == count:
                break
            field = s[k * width:(k + 1) * width].strip()
            if not field:
                break
            out.append(conv(field))
        ln += 1
    return out, ln


def _real(s):
    return float(s.replace("D", "E").replace("d", "e"))


def rb_read(filename, make_values="random", seed=0):
    """Read an assembled Rutherford-Boeing matrix.

    Returns (m, n, ptr, row, val, type_code) with 0-based ptr/row; symmetric
    types give the lower triangle by columns.  For a pattern-only file
    `make_values` chooses made-up values: "random" (uniform[-1,1] entries,
    the reference reader's option 2), "dominant" (random off-diagonals and a
    diagonal of row abs-sum + 1, which makes the matrix positive definite),
    or None (val is None)."""
    with open(filename) as fh:
        lines = fh.readlines()
    if len(lines) < 4:
        raise ValueError("not a Rutherford-Boeing file (short header)")
    type_code = lines[2][:3].lower()
    if type_code[0] not in "rcipq" or type_code[1] not in "suhzr":
        raise ValueError(f"not a Rutherford-Boeing file (type code {type_code!r})")
    if type_code[0] == "c":
        raise ValueError("complex matrices are not supported")
    if type_code[2] != "a":
        raise ValueError("only assembled matrices are supported")
    nums = [int(x) for x in lines[2][3:].split()]
    m, n, nnz = nums[0], nums[1], nums[2]
    fmts = lines[3]
    ptrfmt, indfmt = fmts[0:16], fmts[16:32]
    valfmt = fmts[32:52] if len(fmts) > 32 else ""
    ptr, ln = _read_fields(lines, 4, n + 1, ptrfmt, int)
    row, ln = _read_fields(lines, ln, nnz, indfmt, int)
    ptr = np.asarray(ptr, dtype=np.int64) - 1
    row = np.asarray(row, dtype=np.int64) - 1
    if type_code[0] in "ri" and valfmt.strip():
        val, ln = _read_fields(lines, ln, nnz, valfmt, _real)
        val = np.asarray(val, dtype=np.float64)
    elif make_values is None:
        val = None
    else:
        rng = np.random.default_rng(seed)
        val = rng.uniform(-1.0, 1.0, nnz)
        if make_values == "dominant":
            cols = np.repeat(np.arange(n), np.diff(ptr))
            diag = row == cols
            a = np.abs(np.where(diag, 0.0, val))
            rs = np.zeros(n)
            np.add.at(rs, row, a)
            if type_code[1] in "sh":
                np.add.at(rs, cols, a)
            val[diag] = rs[row[diag]] + 1.0
    return m, n, ptr, row, val, type_code


def rb_write(filename, ptr, row, val, type_code="rsa", title="", identifier="spral"):
    """Write an assembled matrix (0-based ptr/row; lower triangle by columns
    for symmetric types) in Rutherford-Boeing format."""
    ptr = np.asarray(ptr, dtype=np.int64)
    row = np.asarray(row, dtype=np.int64)
    n = len(ptr) - 1
    nnz = int(ptr[-1])
    m = int(row.max()) + 1 if nnz else n
    if type_code[1] in "sh":
        m = n
    iw = max(len(str(max(nnz + 1, m, 1))) + 1, 2)
    iper = max(80 // iw, 1)
    vw, vper = 26, 3
    ipfmt = f"({iper}I{iw})"
    vfmt = f"(3E{vw}.16)"

    def block(vals, per, fmt):
        out = []
        for i in range(0, len(vals), per):
            out.append("".join(fmt(v) for v in vals[i:i + per]))
        return out

    pl = block(list(ptr + 1), iper, lambda v: f"{int(v):{iw}d}")
    rl = block(list(row + 1), iper, lambda v: f"{int(v):{iw}d}")
    vl = [] if val is None or type_code[0] == "p" else \
        block(list(np.asarray(val, dtype=np.float64)), vper, lambda v: f"{v:{vw}.16E}")
    with open(filename, "w") as fh:
        fh.write(f"{title[:72]:<72}{identifier[:8]:<8}\n")
        fh.write(f"{len(pl) + len(rl) + len(vl):14d}{len(pl):14d}{len(rl):14d}{len(vl):14d}\n")
        fh.write(f"{type_code:<3}{'':11}{m:14d}{n:14d}{nnz:14d}{0:14d}\n")
        fh.write(f"{ipfmt:<16}{ipfmt:<16}{vfmt if vl else '':<20}\n")
        for ln in pl + rl + vl:
            fh.write(ln + "\n")
