"""Input files and output parsers for BLIS's own test programs (testsuite, netlib BLAS tests).

The programs are the reference's, compiled by oracle/ref_blis.py and linked
GPU-backed by integration/build.py; this module only writes their parameter
files (the formats the programs read: testsuite/src/test_libblis.c
libblis_test_read_params_file / libblis_test_read_ops_file, and the netlib
?blat?.in layout of blastest/src/?blat?.c) and reads back their verdicts.
"""
import os
import re
import subprocess

# testsuite operations in the order test_libblis.c reads them, with the number of
# dimension specifiers and parameter characters of each (test_libblis.c:398-470)
TS_OPS = [
    ("randv", 1, 0), ("randm", 2, 0),
    ("addv", 1, 1), ("amaxv", 1, 0), ("axpbyv", 1, 1), ("axpyv", 1, 1), ("copyv", 1, 1),
    ("dotv", 1, 2), ("dotxv", 1, 2), ("normfv", 1, 0), ("invscalv", 1, 1), ("scalv", 1, 1),
    ("scal2v", 1, 1), ("setv", 1, 0), ("subv", 1, 1), ("xpbyv", 1, 1),
    ("addm", 2, 1), ("axpym", 2, 1), ("copym", 2, 1), ("normfm", 2, 0), ("invscalm", 2, 1),
    ("scalm", 2, 1), ("scal2m", 2, 1), ("setm", 2, 0), ("subm", 2, 1), ("xpbym", 2, 1),
    ("axpy2v", 1, 2), ("dotaxpyv", 1, 3), ("axpyf", 2, 2), ("dotxf", 2, 2), ("dotxaxpyf", 2, 4),
    ("gemv", 2, 2), ("ger", 2, 2), ("hemv", 1, 3), ("her", 1, 2), ("her2", 1, 3), ("symv", 1, 3),
    ("syr", 1, 2), ("syr2", 1, 3), ("trmv", 1, 3), ("trsv", 1, 3),
    ("gemm_ukr", 1, 0), ("gemmsup_ukr", 1, 0), ("trsm_ukr", 0, 1), ("gemmtrsm_ukr", 1, 1),
    ("gemm", 3, 2), ("gemmt", 2, 3), ("hemm", 2, 4), ("herk", 2, 2), ("her2k", 2, 3),
    ("symm", 2, 4), ("syrk", 2, 2), ("syr2k", 2, 3), ("trmm", 2, 4), ("trmm3", 2, 5), ("trsm", 2, 4),
]
# dimension specifiers used for the operations enabled here (-1: the problem size,
# -2: half of it), as in the reference's own input.operations
TS_DIMS = {"axpyv": "-1", "dotv": "-1", "gemv": "-1 -2", "gemm": "-1 -1 -1", "trsm": "-1 -1"}


def write_testsuite_inputs(dirpath, ops, datatypes, rand_method, sizes=(100, 300, 100),
                           storage="rcg", vstorage="cj"):
    """Writes input.general / input.operations enabling only `ops` (switch 2) and
    returns their paths."""
    gen = os.path.join(dirpath, "input.general")
    lines = [
        "1       # repeats",
        "%-7s # matrix storage schemes" % storage,
        "%-7s # vector storage schemes" % vstorage,
        "0       # all storage combinations",
        "1       # aligned buffers",
        "%d       # randomisation: 0 real on [-1,1], 1 narrow powers of two" % rand_method,
        "32      # general stride spacing",
        "%-7s # datatypes" % datatypes,
        "0       # mixed domain",
        "0       # mixed precision",
        "%d     # first problem size" % sizes[0],
        "%d     # largest problem size" % sizes[1],
        "%d     # increment" % sizes[2],
        "1       # 1m",
        "1       # native",
        "1       # testsuite threads",
        "1       # error checking",
        "i       # on failure: ignore",
        "0       # matlab output",
        "0       # output to files too",
    ]
    with open(gen, "w") as f:
        f.write("\n".join(lines) + "\n")
    opf = os.path.join(dirpath, "input.operations")
    out = ["1 # section override"] * 7
    for name, ndims, npar in TS_OPS:
        out.append("%d # %s" % (2 if name in ops else 0, name))
        if ndims:
            out.append(TS_DIMS.get(name, " ".join(["-1"] * ndims)) + " # dims")
        if npar:
            out.append("?" * npar + " # params")
    with open(opf, "w") as f:
        f.write("\n".join(out) + "\n")
    return gen, opf


TS_LINE = re.compile(r"^blis_([sdcz])(\w+?)_(\S+)\s+.*\s(PASS|MARGINAL|FAILURE|FAIL)\s*$")


def parse_testsuite(text):
    """{(dt, op): {"PASS": n, "MARGINAL": n, "FAIL": n}} from the testsuite's stdout."""
    res = {}
    for ln in text.splitlines():
        m = TS_LINE.match(ln.strip())
        if not m:
            continue
        dt, rest, verdict = m.group(1), m.group(2) + "_" + m.group(3), m.group(4)
        op = rest.split("_")[0]
        v = "FAIL" if verdict.startswith("FAIL") else verdict
        res.setdefault((dt, op), {"PASS": 0, "MARGINAL": 0, "FAIL": 0})[v] += 1
    return res


def parse_report(stderr):
    """Counts printed by libgb300_blis.so at exit (GB300_BLIS_REPORT=1), as a dict."""
    m = re.search(r"gb300_blis: (.*)", stderr)
    if not m:
        return None
    return {k: int(v) for k, v in re.findall(r"(\w+)=(-?\d+)", m.group(1))}


# ---------------------------------------------------------------- netlib BLAS tests
def _blat_header(prog, thresh=16.0):
    return ["'out.%s'          NAME OF SUMMARY OUTPUT FILE" % prog,
            "6                 UNIT NUMBER OF SUMMARY FILE",
            "'%s.SNAP'         NAME OF SNAPSHOT OUTPUT FILE" % prog.upper(),
            "-1                UNIT NUMBER OF SNAPSHOT FILE (NOT USED IF .LT. 0)",
            "F        LOGICAL FLAG, T TO REWIND SNAPSHOT FILE AFTER EACH RECORD.",
            "F        LOGICAL FLAG, T TO STOP ON FAILURES.",
            "T        LOGICAL FLAG, T TO TEST ERROR EXITS.",
            "%.1f     THRESHOLD VALUE OF TEST RATIO" % thresh]


def blat_input(prog, params):
    """The ?blat2 / ?blat3 parameter file, from the values in tests/golden/blastest_params.json
    (extracted from the reference's dblat2.in / dblat3.in); complex programs take the
    real values as complex numbers with a nonzero imaginary part for the third."""
    ch = prog[0]
    level = prog[-1]
    cplx = ch in "zc"
    p = params["dblat%s" % level]

    def scal(vals, imag):
        if not cplx:
            return " ".join(repr(float(v)) for v in vals)
        out = []
        for i, v in enumerate(vals):
            out.append("(%s,%s)" % (float(v), imag if i == len(vals) - 1 else 0.0))
        return " ".join(out)

    lines = _blat_header(prog, p["thresh"])
    lines += ["%d                 NUMBER OF VALUES OF N" % len(p["n"]),
              " ".join(str(v) for v in p["n"]) + "       VALUES OF N"]
    if level == "2":
        lines += ["%d                 NUMBER OF VALUES OF K" % len(p["k"]),
                  " ".join(str(v) for v in p["k"]) + "       VALUES OF K",
                  "%d                 NUMBER OF VALUES OF INCX AND INCY" % len(p["inc"]),
                  " ".join(str(v) for v in p["inc"]) + "       VALUES OF INCX AND INCY"]
    lines += ["%d                 NUMBER OF VALUES OF ALPHA" % len(p["alpha"]),
              scal(p["alpha"], -0.9) + "       VALUES OF ALPHA",
              "%d                 NUMBER OF VALUES OF BETA" % len(p["beta"]),
              scal(p["beta"], -1.1) + "       VALUES OF BETA"]
    up = ch.upper()
    if level == "3":
        names = ["GEMM", "HEMM", "SYMM", "TRMM", "TRSM", "HERK", "SYRK", "HER2K", "SYR2K"] if cplx else \
                ["GEMM", "SYMM", "TRMM", "TRSM", "SYRK", "SYR2K"]
    else:
        names = ["GEMV", "GBMV", "HEMV", "HBMV", "HPMV", "TRMV", "TBMV", "TPMV", "TRSV", "TBSV", "TPSV",
                 "GERC", "GERU", "HER", "HPR", "HER2", "HPR2"] if cplx else \
                ["GEMV", "GBMV", "SYMV", "SBMV", "SPMV", "TRMV", "TBMV", "TPMV", "TRSV", "TBSV", "TPSV",
                 "GER", "SYR", "SPR", "SYR2", "SPR2"]
    lines += ["%-6s T PUT F FOR NO TEST. SAME COLUMNS." % (up + nm) for nm in names]
    return "\n".join(lines) + "\n"


BLAT_VERDICT = re.compile(r"^\s*(\w+)\s+(PASSED|FAILED|\*\*\*)", re.M)


def run_blat(binpath, prog, workdir, params, env=None, timeout=900):
    """Runs one netlib BLAS test program; returns (returncode, summary text, stderr)."""
    os.makedirs(workdir, exist_ok=True)
    exe = os.path.abspath(os.path.join(binpath, prog + ".x"))
    stdin = None
    if prog[-1] in "23":
        stdin = blat_input(prog, params)
    r = subprocess.run([exe], input=stdin, capture_output=True, text=True, cwd=workdir, env=env,
                       timeout=timeout)
    summary = r.stdout
    out = os.path.join(workdir, "out." + prog)
    if os.path.exists(out):
        summary += open(out).read()
    return r.returncode, summary, r.stderr


def blat_results(summary):
    """{routine: set of verdict words} from a ?blat2/3 summary; level-1 programs print
    '----- PASS -----' / '----- FAIL -----' after each subprogram's name."""
    res = {}
    for m in re.finditer(r"^\s*([SDCZI][A-Z0-9]+)\s+PASSED THE (COMPUTATIONAL TESTS|TESTS OF ERROR-EXITS)",
                         summary, re.M):
        res.setdefault(m.group(1), set()).add("PASSED " + m.group(2))
    for m in re.finditer(r"^\s*([SDCZI][A-Z0-9]+)\s+FAILED", summary, re.M):
        res.setdefault(m.group(1), set()).add("FAILED")
    for m in re.finditer(r"Test of subprogram number\s+\d+\s+(\w+)\s*\n\s*-+\s*(PASS|FAIL)", summary):
        res.setdefault(m.group(1), set()).add(m.group(2))
    if re.search(r"\*\*\*\*\*\*", summary):
        res.setdefault("_", set()).add("ERROR")
    return res
