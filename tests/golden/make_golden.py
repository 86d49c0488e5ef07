"""Regenerates the golden fixtures of this directory from the reference's own
test inputs, read as text (nothing of the reference is compiled or run).

  dblat1_check2.json  DDOT / DAXPY known answers of the netlib level-1 test
                      driver (blastest/src/dblat1.c, check2_: data at
                      :411-431, loop at :590-660)
  blastest_params.json the N / ALPHA / BETA / K / INC values and the test-ratio
                      threshold of blastest/input/dblat2.in and dblat3.in

Usage: python tests/golden/make_golden.py PATH-TO-REFERENCE-TREE
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def _array(src, name, cast=float):
    m = re.search(r"static\s+\w+\s+%s\[\d+\][^=]*=\s*\{([^}]*)\}" % re.escape(name), src)
    if not m:
        raise ValueError("array %s not found" % name)
    body = re.sub(r"/\*.*?\*/", "", m.group(1), flags=re.S)
    return [cast(v.strip().rstrip("f")) for v in body.split(",") if v.strip()]


def _scalar(src, name):
    m = re.search(r"static\s+doublereal\s+%s\s*=\s*([-0-9.eE+]+)\s*;" % re.escape(name), src)
    return float(m.group(1))


def dblat1(ref):
    src = open(os.path.join(ref, "blastest", "src", "dblat1.c")).read()
    start = src.index("int check2_(")
    chk = src[start:src.index("} /* check2_ */", start)]
    out = {
        "source": "blastest/src/dblat1.c check2_",
        "sfac": _scalar(src, "sfac"),
        "sa": _scalar(chk, "sa"),
        "incxs": _array(chk, "incxs", int),
        "incys": _array(chk, "incys", int),
        "lens": _array(chk, "lens", int),       # [4][2] Fortran order: lens(kn, mx)
        "ns": _array(chk, "ns", int),
        "dx1": _array(chk, "dx1"),
        "dy1": _array(chk, "dy1"),
        "dt7": _array(chk, "dt7"),              # [4][4]: dt7(kn, ki)
        "dt8": _array(chk, "dt8"),              # [7][4][4]: dt8(j, kn, ki)
        "ssize1": _array(chk, "ssize1"),
        "ssize2": _array(chk, "ssize2"),        # [14][2]
    }
    return out


def _numbers(line):
    return [float(v) for v in line.split()[:64] if re.fullmatch(r"[-+]?[0-9.]+(e[-+]?\d+)?", v, re.I)]


def blastest_inputs(ref):
    res = {}
    for name in ("dblat2", "dblat3"):
        lines = open(os.path.join(ref, "blastest", "input", name + ".in")).read().splitlines()
        rec = {"source": "blastest/input/%s.in" % name}
        for ln in lines:
            key = ln.split("  ")[-1].strip() if "  " in ln else ""
            vals = ln.split()
            if "THRESHOLD VALUE" in ln:
                rec["thresh"] = float(vals[0])
            elif "VALUES OF N" in ln:
                rec["n"] = [int(v) for v in vals if v.isdigit()]
            elif "VALUES OF K" in ln:
                rec["k"] = [int(v) for v in vals if v.isdigit()]
            elif "VALUES OF INCX" in ln:
                rec["inc"] = [int(v) for v in vals if re.fullmatch(r"-?\d+", v)]
            elif "VALUES OF ALPHA" in ln:
                rec["alpha"] = _numbers(ln)
            elif "VALUES OF BETA" in ln:
                rec["beta"] = _numbers(ln)
            del key
        res[name] = rec
    return res


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py PATH-TO-REFERENCE-TREE")
    ref = sys.argv[1]
    with open(os.path.join(HERE, "dblat1_check2.json"), "w") as f:
        json.dump(dblat1(ref), f, indent=1)
    with open(os.path.join(HERE, "blastest_params.json"), "w") as f:
        json.dump(blastest_inputs(ref), f, indent=1)
    print("wrote fixtures to", HERE)


if __name__ == "__main__":
    main()
