"""Times the reference's own host partitioner (TEST INFRASTRUCTURE ONLY).

Runs oracle/_ref/ref_partition_harness (built by oracle/build_ref.sh from the
reference sources, Xilinx/HPC L2/sparse/src/sw/c++/gen_signature.cpp) on the
27-point variable-coefficient diffusion matrix of a given grid, with the COO
entries in a seeded random order, and prints the wall time of the partition
call alone (SpmPar::partitionCooMat, gen_signature.hpp:41-73) with its OpenMP
thread count.  This is the format-conversion baseline that the GPU exporter
(xJPCG_gbExportSignature) and the solver's device COO-to-CSR conversion are
compared with.  The harness is an x86 build of the reference: it runs where
the reference sources are, not on the GPU host.

Usage: python oracle/time_ref_partition.py [nx] [work-dir]
"""
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))


def main():
    from hpc_gb300 import workloads as W
    nx = int(sys.argv[1]) if len(sys.argv) > 1 else 160
    work = sys.argv[2] if len(sys.argv) > 2 else tempfile.mkdtemp(prefix="refpart")
    harness = os.path.join(HERE, "_ref", "ref_partition_harness")
    if not os.path.exists(harness):
        raise SystemExit("build the harness first: sh oracle/build_ref.sh")
    s = W.diffusion27(nx)
    r, c, v = s.coo()
    perm = np.random.default_rng(0).permutation(len(r))
    os.makedirs(work, exist_ok=True)
    with open(os.path.join(work, "meta.txt"), "w") as f:
        f.write("%d %d\n" % (s.n, s.nnz))
    r[perm].astype(np.uint32).tofile(os.path.join(work, "row.bin"))
    c[perm].astype(np.uint32).tofile(os.path.join(work, "col.bin"))
    v[perm].astype(np.float64).tofile(os.path.join(work, "data.bin"))
    del r, c, v, perm
    try:
        p = subprocess.run([harness, "coo", work, "0"], capture_output=True, text=True)
        if p.returncode != 0:
            raise SystemExit("harness failed (%d): %s" % (p.returncode, p.stderr[-500:]))
        with open(os.path.join(work, "ref_time.txt")) as f:
            sec, threads = f.read().split()
        print("27-point %d^3: n=%d nnz=%d reference partitionCooMat %.2f s on %s OpenMP threads" %
              (nx, s.n, s.nnz, float(sec), threads))
    finally:
        if len(sys.argv) <= 2:
            shutil.rmtree(work, ignore_errors=True)


if __name__ == "__main__":
    main()
