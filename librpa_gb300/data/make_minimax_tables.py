"""Extract the GreenX minimax coefficient tables into a plain data file.

The tabulated minimax points/weights for the imaginary-time and
imaginary-frequency quadratures live, as Fortran array literals, in the GreenX
library that LibRPA vendors (thirdparty/greenX/GX-TimeFrequency/src/
minimax_omega.F90 and minimax_tau.F90, Apache-2.0, Copyright (C) 2020-2023
GreenX library).  They are numeric data, not code: this script copies the
numbers verbatim (same decimal strings) into ``greenx_minimax_tables.txt`` so
the host grid generator can read them at run time without a Fortran compiler.

Usage:  python make_minimax_tables.py <path to GX-TimeFrequency/src> [out]

Output format (whitespace separated, one record per line):
    table <omega|tau> <num_points> <n_ranges>
    erange <n_ranges values>
    col <index 1..n_ranges+1> <2*num_points values>
"""
import re
import sys
from pathlib import Path

_NUM = re.compile(r"([-+]?[0-9]*\.?[0-9]+(?:[eEdD][-+]?[0-9]+)?)_dp")


def _statements(text):
    """Join Fortran '&' continuation lines into single statements."""
    out, cur = [], ""
    for raw in text.splitlines():
        line = raw.split("!")[0].rstrip()
        if not line.strip():
            continue
        if cur:
            cur += " " + line.strip().lstrip("&")
        else:
            cur = line.strip()
        if cur.endswith("&"):
            cur = cur[:-1]
            continue
        out.append(cur)
        cur = ""
    if cur:
        out.append(cur)
    return out


def parse(path, kind):
    text = Path(path).read_text()
    stmts = _statements(text)
    tables = {}
    current = None
    for s in stmts:
        m = re.match(r"case\s*\(\s*(\d+)\s*\)", s)
        if m:
            current = int(m.group(1))
            tables[current] = {"erange": None, "cols": {}}
            continue
        if current is None:
            continue
        if s.startswith("aw%energy_range"):
            tables[current]["erange"] = _NUM.findall(s)
        m = re.match(r"aw%aw_erange_matrix\(:,\s*(\d+)\)", s)
        if m:
            tables[current]["cols"][int(m.group(1))] = _NUM.findall(s)
        if s.startswith("end select"):
            current = None
    out = []
    for n in sorted(tables):
        t = tables[n]
        nr = len(t["erange"])
        assert len(t["cols"]) == nr + 1, (kind, n, len(t["cols"]), nr)
        for k, v in t["cols"].items():
            assert len(v) == 2 * n, (kind, n, k, len(v))
        out.append(f"table {kind} {n} {nr}")
        out.append("erange " + " ".join(t["erange"]))
        for k in sorted(t["cols"]):
            out.append(f"col {k} " + " ".join(t["cols"][k]))
    return out


def main():
    src = Path(sys.argv[1])
    dst = Path(sys.argv[2]) if len(sys.argv) > 2 else Path(__file__).with_name("greenx_minimax_tables.txt")
    lines = [
        "# Minimax quadrature tables of the GreenX library (GX-TimeFrequency),",
        "# Apache License 2.0, Copyright (C) 2020-2023 GreenX library.",
        "# Numbers copied verbatim from minimax_omega.F90 / minimax_tau.F90 by make_minimax_tables.py.",
    ]
    lines += parse(src / "minimax_omega.F90", "omega")
    lines += parse(src / "minimax_tau.F90", "tau")
    dst.write_text("\n".join(lines) + "\n")
    print(f"wrote {dst} ({len(lines)} lines)")


if __name__ == "__main__":
    main()
