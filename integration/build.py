"""Build recipe: BLIS wired to libblis_gb300.so through its own seams.

Outputs, under integration/_build/<cfg>/ (git-ignored; <cfg> is the CPU
sub-configuration BLIS would pick on this host, see oracle/ref_blis.py):

  lib/libblis.so        BLIS compiled with the gb300 gemm sandbox
                        (integration/sandbox/gb300): its bli_gemm_ex calls the GPU
  lib/libgb300_blis.so  the glue library (integration/gb300_blis.c): bli_trsm_ex and
                        bli_dgemv_ex interposed, axpyv/dotv kernels registered in
                        BLIS's context
  bin/test_libblis.x, bin/?blat?.x
                        BLIS's testsuite and the netlib BLAS tests, unchanged, linked
                        -lgb300_blis -lblis (the sandbox build): every gemm, trsm, gemv,
                        axpyv and dotv they run goes through BLIS's host code to the GPU
  bin_interpose/?blat?.x  the same BLAS tests linked -lblis_gb300 -lblis (plain BLIS):
                        the library's own BLAS front ends interpose BLIS's
  bin/obj_gemm_comp_prec.x
                        a BLIS object-API program (tests/blis/obj_gemm_comp_prec.c) that
                        sends one double gemm with a single-precision computation
                        request through the sandbox

The BLIS sources come from the same place as the reference build's (the
reference tree, or the snapshot oracle/ref_blis.py ships to machines without
it); the testsuite and blastest objects are that build's.  Nothing here runs the
reference's configure or make.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from oracle import ref_blis  # noqa: E402

SANDBOX = os.path.join(HERE, "sandbox", "gb300")
SHIM_SRC = os.path.join(HERE, "gb300_blis.c")
COMP_PREC_SRC = os.path.join(ROOT, "tests", "blis", "obj_gemm_comp_prec.c")
GB_LIB_DIR = os.path.join(ROOT, "blis_gb300")
INCLUDE = os.path.join(ROOT, "include")


def out_dir(cfg=None):
    cfg = cfg or ref_blis.host_config()
    return os.path.join(HERE, "_build", cfg["CFG"])


def paths(cfg=None):
    o = out_dir(cfg)
    return {
        "lib": os.path.join(o, "lib"),
        "bin": os.path.join(o, "bin"),
        "bin_interpose": os.path.join(o, "bin_interpose"),
        "libblis": os.path.join(o, "lib", "libblis.so"),
        "shim": os.path.join(o, "lib", "libgb300_blis.so"),
        "comp_prec": os.path.join(o, "bin", "obj_gemm_comp_prec.x"),
    }


def _rel_rpath(frm, to):
    return "$ORIGIN/" + os.path.relpath(to, frm)


def _inputs_mtime():
    files = [SHIM_SRC, COMP_PREC_SRC, ref_blis.MAKEFILE, os.path.join(INCLUDE, "blis_gb300.h")]
    files += [os.path.join(SANDBOX, f) for f in os.listdir(SANDBOX)]
    return max(os.path.getmtime(f) for f in files)


def build(force=False):
    """Returns the paths dict, or None when no BLIS sources are available."""
    ref_lib = ref_blis.build()
    if ref_lib is None:
        return None
    src = ref_blis.source_root()
    cfg = ref_blis.host_config()
    o = out_dir(cfg)
    p = paths(cfg)
    stamp = os.path.join(o, ".built")
    key = "%s|%s" % (src, _inputs_mtime())
    if (not force and os.path.exists(stamp) and open(stamp).read() == key
            and all(os.path.exists(p[k]) for k in ("libblis", "shim", "comp_prec"))):
        return p

    libdir = p["lib"]
    os.makedirs(libdir, exist_ok=True)
    gb_rpath = _rel_rpath(libdir, GB_LIB_DIR)
    ref_blis.write_config_headers(src, os.path.join(o, "gen"), cfg, sandbox=True)
    ref_blis.run_make(src, o, cfg, ["lib"], sandbox_dir=SANDBOX,
                      extra={"SBOX_CFLAGS": "-I" + INCLUDE,
                             "LIBEXTRA": "-L%s -lblis_gb300 -Wl,-rpath,%s" % (GB_LIB_DIR, gb_rpath)})

    # compile flags of an application of this BLIS tree (blis.h and the sandbox's bli_sandbox.h)
    r = subprocess.run(["make", "-s", "-f", ref_blis.MAKEFILE, "SRC=" + src, "OUT=" + o, "CFG=" + cfg["CFG"],
                        "KSETS=" + cfg["KSETS"], "CPPROC=" + cfg["CPPROC"], "SANDBOX=" + SANDBOX,
                        "print-cflags"], capture_output=True, text=True, check=True)
    cflags = r.stdout.split()

    def cc(args):
        rr = subprocess.run(["gcc"] + args, capture_output=True, text=True)
        if rr.returncode != 0:
            raise RuntimeError("gcc failed: %s\n%s" % (" ".join(args[-6:]), rr.stderr[-3000:]))

    cc(cflags + ["-O2", "-D_GNU_SOURCE", "-I" + INCLUDE, "-shared", SHIM_SRC, "-o", p["shim"],
                 "-L" + libdir, "-lblis", "-L" + GB_LIB_DIR, "-lblis_gb300", "-ldl",
                 "-Wl,-rpath," + _rel_rpath(libdir, libdir), "-Wl,-rpath," + gb_rpath])

    # BLIS's own test programs (objects of the reference build), GPU-backed link order
    ref_out = ref_blis.config_dir(cfg)
    gb_libs = ["-L" + libdir, "-lgb300_blis", "-lblis"]
    ref_blis.link_programs_from(ref_out, gb_libs, p["bin"],
                                ["$ORIGIN/" + os.path.relpath(libdir, p["bin"]),
                                 "$ORIGIN/" + os.path.relpath(GB_LIB_DIR, p["bin"])])
    # and the BLAS tests with the library's BLAS fronts interposed ahead of plain BLIS
    plain_lib = os.path.join(ref_out, "lib")
    ref_blis.link_programs_from(ref_out, ["-L" + GB_LIB_DIR, "-lblis_gb300", "-L" + plain_lib, "-lblis"],
                                p["bin_interpose"],
                                ["$ORIGIN/" + os.path.relpath(GB_LIB_DIR, p["bin_interpose"]),
                                 "$ORIGIN/" + os.path.relpath(plain_lib, p["bin_interpose"])],
                                testsuite=False)
    cc(cflags + ["-O2", "-I" + INCLUDE, COMP_PREC_SRC, "-o", p["comp_prec"], "-Wl,--no-as-needed"] + gb_libs +
       ["-L" + GB_LIB_DIR, "-lblis_gb300",
        "-Wl,-rpath,$ORIGIN/" + os.path.relpath(libdir, p["bin"]),
        "-Wl,-rpath,$ORIGIN/" + os.path.relpath(GB_LIB_DIR, p["bin"]), "-lm", "-lpthread"])
    with open(stamp, "w") as f:
        f.write(key)
    return p


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
