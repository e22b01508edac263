"""Build recipes for the oracle (test infrastructure only).

``build_oracle()`` compiles the C restatement ``oracle/st3d_oracle.c`` into
``oracle/_build/libst3d_oracle.so``.  ``build_ref()`` compiles the reference's
own host path from its sources with ``oracle/Makefile.ref`` into
``oracle/_ref/``; the directory holding the reference's sources is named by
the environment variable ``ST3D_REFERENCE_DIR`` (no default: without it, or
where the sources are absent, nothing is built).
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
ORACLE_SO = os.path.join(HERE, "_build", "libst3d_oracle.so")
REF_DIR = os.path.join(HERE, "_ref")


def ref_source_dir():
    """The reference's source directory (ST3D_REFERENCE_DIR), or None."""
    d = os.environ.get("ST3D_REFERENCE_DIR")
    return d if d and os.path.isfile(os.path.join(d, "iterators.cpp")) else None


def build_oracle(force=False):
    src = os.path.join(HERE, "st3d_oracle.c")
    os.makedirs(os.path.dirname(ORACLE_SO), exist_ok=True)
    if (not force and os.path.exists(ORACLE_SO)
            and os.path.getmtime(ORACLE_SO) >= os.path.getmtime(src)):
        return ORACLE_SO
    cmd = ["gcc", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           "-std=gnu11", "-o", ORACLE_SO, src, "-lm"]
    subprocess.run(cmd, check=True)
    return ORACLE_SO


def build_ref():
    """Compile oracle/_ref from the reference sources; False if they are not given."""
    src = ref_source_dir()
    if src is None:
        return False
    subprocess.run(["make", "-s", "-f", os.path.join(HERE, "Makefile.ref"),
                    "REFDIR=" + src, "OUT=" + REF_DIR, "-j8"],
                   check=True, cwd=REPO)
    return True


if __name__ == "__main__":
    print(build_oracle(force=True))
    print("reference built:", build_ref())
