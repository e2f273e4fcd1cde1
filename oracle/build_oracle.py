"""Builds the CPU checkers.

  * oracle/_build/liborc.so  from oracle/g4oracle.c (always; plain C, no GPU)
  * oracle/_ref/             the reference compiled from its own sources by
                             oracle/ref_build/Makefile, only when a reference
                             source tree is named (argument or G4_REFERENCE_DIR)
                             and present

Test infrastructure: called by __graft_entry__.build() and the tests.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def build_oracle(verbose=False):
    out_dir = os.path.join(HERE, "_build")
    os.makedirs(out_dir, exist_ok=True)
    out = os.path.join(out_dir, "liborc.so")
    src = os.path.join(HERE, "g4oracle.c")
    hdr = os.path.join(HERE, "g4oracle.h")
    if os.path.exists(out) and os.path.getmtime(out) >= max(os.path.getmtime(src), os.path.getmtime(hdr)):
        return out
    # -ffp-contract=off: no fused multiply-add, every operation rounds as in the reference
    cmd = ["gcc", "-std=c11", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-o", out + ".tmp",
           src, "-lm", "-lpthread"]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(out + ".tmp", out)
    return out


def build_reference(ref_dir=None, jobs=8):
    ref_dir = ref_dir or os.environ.get("G4_REFERENCE_DIR")
    if not ref_dir or not os.path.isdir(os.path.join(ref_dir, "src", "Core")):
        return None
    subprocess.check_call(["make", "-s", "-C", os.path.join(HERE, "ref_build"), f"REF={ref_dir}",
                           f"-j{jobs}"])
    return os.path.join(HERE, "_ref", "libg4ref.so")


if __name__ == "__main__":
    print(build_oracle(verbose=True))
    print(build_reference(sys.argv[1] if len(sys.argv) > 1 else None))
    sys.exit(0)
