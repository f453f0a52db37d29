"""Regenerate ``tess_table_nv.bin`` from the reference's tessellation table.

The tessellation patterns are data that must match the reference bit for bit
(the per-config triangle index streams and barycentric vertices are what the
cluster templates and the split tree are built from), so they are taken from
the reference's generated header ``src/tessellation_table_nv_raw.hpp`` rather
than re-derived. The header is compiled unchanged by ``oracle/Makefile`` (target
``ref``) into a small dumper that writes the binary container documented in
``oracle/ref_table_dump.cpp``; this script runs it and copies the result next
to itself.

Usage: python vk_tessellated_clusters_gb300/data/make_tess_table.py [REF_ROOT]
"""
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))


def main() -> int:
    # the checkout: argv[1], else TC_REFERENCE_ROOT, else the oracle recipe's default
    extra = [f"REF_ROOT={sys.argv[1]}"] if len(sys.argv) > 1 else []
    subprocess.check_call(["make", "-C", os.path.join(REPO, "oracle"), "ref"] + extra)
    dumper = os.path.join(REPO, "oracle", "_ref", "ref_table_dump")
    tmp = os.path.join(REPO, "oracle", "_ref", "tess_table_nv.bin")
    subprocess.check_call([dumper, tmp])
    dst = os.path.join(HERE, "tess_table_nv.bin")
    shutil.copyfile(tmp, dst)
    with open(dst, "rb") as f:
        print("sha256", hashlib.sha256(f.read()).hexdigest())
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
