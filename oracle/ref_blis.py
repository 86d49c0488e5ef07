"""Recipe: the reference BLIS, compiled from its own C sources (test infrastructure only).

What it builds, all under oracle/_ref/ (git-ignored):
  blis-src.tar.gz   a snapshot of the BLIS source files the build needs, taken from the
                    reference tree (/root/reference) in the container that has it; the
                    GPU machine has no reference tree, so it compiles from this snapshot
  src/              the snapshot unpacked (on machines without the reference tree)
  <cfg>/lib/libblis.so          BLIS itself, plain (no sandbox), for the CPU sub-configuration
                                BLIS's configure would pick on this machine ("auto"): haswell on
                                x86-64, armsve on an aarch64 core with SVE (bli_cpuid.c sends every
                                SVE part it does not list to armsve), cortexa57 without SVE
  <cfg>/bin/test_libblis.x      the BLIS testsuite linked against it
  <cfg>/bin/?blat?.x            the netlib BLAS tests (f2c'd) linked against it
  <cfg>/lib/libf2c.a, obj/      intermediates

It never runs the reference's configure or make: oracle/blis.mk compiles the sources with
gcc, and this script writes the two configuration headers (bli_config.h, bli_addon.h) from
the source tree's own templates with the values of a `configure -t pthreads --enable-cblas
auto` build.  Nothing under blis_gb300/ links or loads any of this; the tests, the oracle
pins and bench.py's CPU legs do.

Usage: python -m oracle.ref_blis [--force]
"""
import os
import platform
import re
import shutil
import subprocess
import sys
import tarfile

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
SNAPSHOT = os.path.join(REF_DIR, "blis-src.tar.gz")
UNPACKED = os.path.join(REF_DIR, "src")
MAKEFILE = os.path.join(HERE, "blis.mk")
REFERENCE_TREE = os.environ.get("GB_BLIS_SRC", "/root/reference")

# Flag sets of the sub-configuration `auto` picks on each host (config/<cfg>/make_defs.mk).
CONFIGS = {
    "x86_64": {
        "CFG": "haswell", "KSETS": "haswell zen",
        "COPT": "-O2", "CKOPT": "-O2 -O3 -fomit-frame-pointer",
        "CKVEC": "-mavx2 -mfma -mfpmath=sse -march=haswell",
        "CRVEC": "-mavx2 -mfma -mfpmath=sse -march=haswell -funsafe-math-optimizations -ffp-contract=fast",
        "CPPROC": "",
    },
    "aarch64-sve": {
        "CFG": "armsve", "KSETS": "armsve",
        "COPT": "-O3 -ftree-vectorize -march=armv8-a+sve",
        "CKOPT": "-O3 -ftree-vectorize -march=armv8-a+sve",
        "CKVEC": "",
        "CRVEC": "-funsafe-math-optimizations -ffp-contract=fast",
        "CPPROC": "-D_GNU_SOURCE",
    },
    # an Arm core without SVE that bli_cpuid.c does not list falls through to cortexa57
    "aarch64": {
        "CFG": "cortexa57", "KSETS": "armv8a",
        "COPT": "-O2 -mcpu=cortex-a57",
        "CKOPT": "-O2 -mcpu=cortex-a57 -O3 -ftree-vectorize",
        "CKVEC": "-mcpu=cortex-a57",
        "CRVEC": "-mcpu=cortex-a57 -funsafe-math-optimizations -ffp-contract=fast",
        "CPPROC": "-D_GNU_SOURCE",
    },
}
CONFIGS["AMD64"] = CONFIGS["x86_64"]

# Subtrees the compile needs (plus the testsuite and blastest inputs).
SNAPSHOT_PATHS = ["frame", "ref_kernels", "config", "kernels/haswell", "kernels/zen",
                  "kernels/armsve", "kernels/armv8a", "testsuite/src", "blastest/f2c", "blastest/src",
                  "blastest/input", "build/bli_config.h.in", "build/bli_addon.h.in",
                  "build/version", "LICENSE"]
for _f in ("input.general", "input.general.fast", "input.operations", "input.operations.fast"):
    SNAPSHOT_PATHS.append("testsuite/" + _f)

BLAST_PROGRAMS = ["dblat1", "dblat2", "dblat3", "sblat1", "sblat2", "sblat3",
                  "zblat1", "zblat2", "zblat3", "cblat1", "cblat2", "cblat3"]


def _cpu_has_sve():
    try:
        with open("/proc/cpuinfo") as f:
            for ln in f:
                if ln.lower().startswith("features"):
                    return "sve" in ln.split(":", 1)[1].split()
    except OSError:
        pass
    return False


def host_config():
    """BLIS's `auto` choice for this host (frame/base/bli_cpuid.c): haswell on this x86-64
    (cpuid cannot count its FMA units), armsve on an Arm core with SVE that it does not list
    by part number (Grace's Neoverse V2), cortexa57 on one without SVE."""
    m = platform.machine()
    if m in ("aarch64", "arm64"):
        m = "aarch64-sve" if _cpu_has_sve() else "aarch64"
    if m not in CONFIGS:
        raise RuntimeError("no BLIS sub-configuration for host %s" % m)
    return dict(CONFIGS[m])


def _ignored(name):
    parts = name.split("/")
    return any(p in ("attic", "old", "broken", "temp", "tmp") for p in parts)


def make_snapshot(force=False):
    """Writes blis-src.tar.gz from the reference tree; returns its path or None."""
    if not os.path.isdir(os.path.join(REFERENCE_TREE, "frame")):
        return SNAPSHOT if os.path.exists(SNAPSHOT) else None
    listing = SNAPSHOT + ".paths"
    want = "\n".join(SNAPSHOT_PATHS)
    if (os.path.exists(SNAPSHOT) and not force and os.path.exists(listing)
            and open(listing).read() == want):
        return SNAPSHOT
    os.makedirs(REF_DIR, exist_ok=True)
    tmp = SNAPSHOT + ".tmp%d" % os.getpid()
    with tarfile.open(tmp, "w:gz", compresslevel=6) as tf:
        for rel in SNAPSHOT_PATHS:
            full = os.path.join(REFERENCE_TREE, rel)
            if not os.path.exists(full):
                continue
            tf.add(full, arcname=rel, filter=lambda ti: None if _ignored(ti.name) else ti)
    os.replace(tmp, SNAPSHOT)
    with open(listing, "w") as f:
        f.write(want)
    return SNAPSHOT


def source_root():
    """The BLIS tree to compile: the reference tree where it exists, else the unpacked snapshot."""
    if os.path.isdir(os.path.join(REFERENCE_TREE, "frame")):
        return REFERENCE_TREE
    if not os.path.exists(SNAPSHOT):
        return None
    stamp = os.path.join(UNPACKED, ".snapshot_mtime")
    want = str(os.path.getmtime(SNAPSHOT))
    if not (os.path.exists(stamp) and open(stamp).read() == want):
        if os.path.isdir(UNPACKED):
            shutil.rmtree(UNPACKED)
        os.makedirs(UNPACKED)
        with tarfile.open(SNAPSHOT, "r:gz") as tf:
            tf.extractall(UNPACKED)
        with open(stamp, "w") as f:
            f.write(want)
    return UNPACKED


def write_config_headers(src, gen, cfg, sandbox=False):
    """bli_config.h / bli_addon.h from the source tree's templates (the values a
    `-t pthreads --enable-cblas auto` configure writes; sandbox on request)."""
    os.makedirs(gen, exist_ok=True)
    ver = open(os.path.join(src, "build", "version")).read().strip()
    mver = re.match(r"(\d+)\.(\d+)(?:\.(\d+))?", ver)
    major, minor, rev = mver.group(1), mver.group(2), mver.group(3) or "0"
    kern = " ".join("#define BLIS_KERNELS_%s\n" % k.upper() for k in cfg["KSETS"].split())
    vals = {
        "config_name_define": "#define BLIS_FAMILY_%s\n" % cfg["CFG"].upper(),
        "config_list_defines": "#define BLIS_CONFIG_%s\n" % cfg["CFG"].upper(),
        "kernel_list_defines": kern.replace("\n ", "\n"),
        "omit_symbol_list_defines": "",
        "version": ver, "version_major": major, "version_minor": minor, "version_revision": rev,
        "enable_system": "1", "enable_tls": "1", "enable_openmp": "0", "enable_openmp_as_def": "0",
        "enable_pthreads": "1", "enable_pthreads_as_def": "1", "enable_hpx": "0",
        "enable_hpx_as_def": "0", "enable_jrir_slab": "1", "enable_jrir_rr": "0",
        "enable_jrir_tlb": "0", "enable_pba_pools": "1", "enable_sba_pools": "1",
        "enable_mem_tracing": "0", "enable_scalapack_compat": "0", "int_type_size": "0",
        "blas_int_type_size": "32", "enable_blas": "1", "enable_cblas": "1",
        "enable_sup_handling": "1", "enable_memkind": "0", "enable_trsm_preinversion": "1",
        "enable_pragma_omp_simd": "1", "enable_sandbox": "1" if sandbox else "0",
        "enable_shared": "1", "complex_return_intel": "0",
    }

    def subst(template, out, table):
        text = open(template).read()

        def rep(mt):
            key = mt.group(1)
            if key not in table:
                raise RuntimeError("unknown template key @%s@ in %s" % (key, template))
            return table[key]
        text = re.sub(r"@([a-z_0-9]+)@", rep, text)
        tmp = out + ".tmp"
        with open(tmp, "w") as f:
            f.write(text)
        if not (os.path.exists(out) and open(out).read() == text):
            os.replace(tmp, out)
        else:
            os.remove(tmp)

    subst(os.path.join(src, "build", "bli_config.h.in"), os.path.join(gen, "bli_config.h"), vals)
    subst(os.path.join(src, "build", "bli_addon.h.in"), os.path.join(gen, "bli_addon.h"),
          {"enable_addons": "0", "addon_list_includes": ""})


def run_make(src, out, cfg, targets, sandbox_dir=None, extra=None, jobs=None):
    jobs = jobs or (os.cpu_count() or 4)
    cmd = ["make", "-s", "-f", MAKEFILE, "-j%d" % jobs, "SRC=" + src, "OUT=" + out]
    for key in ("CFG", "KSETS", "COPT", "CKOPT", "CKVEC", "CRVEC", "CPPROC"):
        cmd.append("%s=%s" % (key, cfg[key]))
    cmd.append("CROPT=" + cfg["CKOPT"])
    if sandbox_dir:
        cmd.append("SANDBOX=" + sandbox_dir)
    for k, v in (extra or {}).items():
        cmd.append("%s=%s" % (k, v))
    cmd += targets
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("BLIS compile failed (%s):\n%s\n%s" % (" ".join(targets), r.stdout[-4000:],
                                                                  r.stderr[-4000:]))


def link_programs_from(out, libs, bindir, rpaths, testsuite=True):
    """Links the testsuite (optional) and the ?blat? programs compiled in the tree `out`
    against `libs` (linker arguments, in link order), with run paths `rpaths`
    ($ORIGIN-relative, so the tree can move)."""
    os.makedirs(bindir, exist_ok=True)
    obj = os.path.join(out, "obj")
    rp = ["-Wl,-rpath," + p for p in rpaths] + ["-Wl,--no-as-needed"]
    cmds = []
    if testsuite:
        ts = sorted(os.path.join(obj, "testsuite", f) for f in os.listdir(os.path.join(obj, "testsuite"))
                    if f.endswith(".o"))
        cmds.append(["gcc", "-o", os.path.join(bindir, "test_libblis.x")] + ts + rp + libs + ["-lm", "-lpthread"])
    f2c = os.path.join(out, "lib", "libf2c.a")
    for p in BLAST_PROGRAMS:
        o = os.path.join(obj, "blastest", "src", p + ".o")
        if os.path.exists(o):
            cmds.append(["gcc", "-o", os.path.join(bindir, p + ".x"), o, f2c] + rp + libs + ["-lm", "-lpthread"])
    for c in cmds:
        r = subprocess.run(c, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s" % (" ".join(c), r.stderr[-3000:]))


def config_dir(cfg=None):
    cfg = cfg or host_config()
    return os.path.join(REF_DIR, cfg["CFG"])


def lib_path(cfg=None):
    return os.path.join(config_dir(cfg), "lib", "libblis.so")


def build(force=False):
    """Builds plain BLIS + its testsuite and blastest programs; returns the library path,
    or None when neither the reference tree nor a snapshot is present."""
    make_snapshot()
    src = source_root()
    if src is None:
        return None
    cfg = host_config()
    out = config_dir(cfg)
    lib = lib_path(cfg)
    stamp = os.path.join(out, ".built")
    key = "%s|%s" % (src, os.path.getmtime(MAKEFILE))
    if not force and os.path.exists(stamp) and open(stamp).read() == key and os.path.exists(lib):
        return lib
    write_config_headers(src, os.path.join(out, "gen"), cfg)
    run_make(src, out, cfg, ["lib", "testsuite", "blastest"])
    libdir = os.path.join(out, "lib")
    link_programs_from(out, ["-L" + libdir, "-lblis"], os.path.join(out, "bin"), ["$ORIGIN/../lib"])
    with open(stamp, "w") as f:
        f.write(key)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
