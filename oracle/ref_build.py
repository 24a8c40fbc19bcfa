"""Compile the reference-generated kernels in oracle/_ref/src/<config>/.

TEST INFRASTRUCTURE (see oracle/__init__.py).  For each configuration two
shared libraries go to oracle/_ref/lib/:
  <config>.strict.so    -O2 -fno-fast-math -ffp-contract=off -fopenmp
                        (the FP64 parity oracle; rounding as written)
  <config>.fast.so      -Ofast -fopenmp -funroll-loops [-march=native]
                        (the reference's own flags, cmdline_helper.py:85;
                        the timed CPU baseline)
Sources exist only where oracle/gen_ref.py ran (they are gitignored and
travel with the working tree); nothing happens when they are absent.
"""
import glob
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "_ref", "src")
LIB = os.path.join(HERE, "_ref", "lib")

STRICT = ["-O2", "-fno-fast-math", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared"]
FAST = ["-Ofast", "-fopenmp", "-funroll-loops", "-fPIC", "-shared"]


def _gcc():
    return os.environ.get("CC") or shutil.which("gcc") or "gcc"


def _compile(cfg, flavour):
    d = os.path.join(SRC, cfg)
    out = os.path.join(LIB, "%s.%s.so" % (cfg, flavour))
    src = os.path.join(d, "shim.c")
    deps = glob.glob(os.path.join(d, "*"))
    if os.path.exists(out) and os.path.getmtime(out) >= max(os.path.getmtime(p) for p in deps):
        return out
    flags = STRICT if flavour == "strict" else FAST
    cmd = [_gcc()] + flags + ["-I" + d, src, "-o", out, "-lm"]
    if flavour == "fast":
        r = subprocess.run(cmd[:1] + ["-march=native"] + cmd[1:], capture_output=True, text=True)
        if r.returncode == 0:
            return out
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("gcc failed for %s (%s):\n%s" % (cfg, flavour, r.stderr[-3000:]))
    return out


def configs():
    if not os.path.isdir(SRC):
        return []
    return sorted(c for c in os.listdir(SRC) if os.path.exists(os.path.join(SRC, c, "shim.c")))


MOL_SRC = os.path.join(HERE, "c", "mol_ref.c")
MOL_LIB = os.path.join(LIB, "mol_ref.so")


def build_mol_ref():
    """Our C restatement of the RK4 update and BC application (always built)."""
    os.makedirs(LIB, exist_ok=True)
    if os.path.exists(MOL_LIB) and os.path.getmtime(MOL_LIB) >= os.path.getmtime(MOL_SRC):
        return MOL_LIB
    cmd = [_gcc(), "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", MOL_SRC, "-o", MOL_LIB]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("gcc failed for mol_ref.c:\n" + r.stderr[-3000:])
    return MOL_LIB


def build_if_present(jobs=None):
    build_mol_ref()
    cfgs = configs()
    if not cfgs:
        return []
    os.makedirs(LIB, exist_ok=True)
    work = [(c, f) for c in cfgs for f in ("strict", "fast")]
    with ThreadPoolExecutor(max_workers=jobs or max(2, os.cpu_count() or 2)) as ex:
        return list(ex.map(lambda a: _compile(*a), work))


if __name__ == "__main__":
    import time
    t = time.time()
    print(build_if_present())
    print("%.1f s" % (time.time() - t))
