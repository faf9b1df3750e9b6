"""Makes the snapshot set in tests/golden/plotting_n3_b211/: the driver's
_log.txt and raw/*.h5 files of a two-block, order-3 run
(plotting_n3_b211.params.txt: snapshots at time steps 0, 2 and 4), which
tests/test_plotting_script.py feeds to the reference's plotting.py.

Needs a GPU and a built driver (``__graft_entry__.build()``):

    python tests/golden/make_plotting_fixture.py <output folder>
"""
import os
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def main(dest: str) -> None:
    exe = os.path.join(ROOT, "3ddg_gb300", "bin", "dg3d")
    with tempfile.TemporaryDirectory() as d:
        for f in ("hardcoded_coeff.txt", "hardcoded_coeff2.txt", "matrices.txt"):
            shutil.copy(os.path.join(HERE, f), d)
        shutil.copy(os.path.join(HERE, "plotting_n3_b211.params.txt"), os.path.join(d, "params.txt"))
        subprocess.run([exe, "params.txt", "results"], cwd=d, check=True)
        os.makedirs(os.path.join(dest, "raw"), exist_ok=True)
        shutil.copy(os.path.join(d, "results", "_log.txt"), dest)
        for f in sorted(os.listdir(os.path.join(d, "results", "raw"))):
            shutil.copy(os.path.join(d, "results", "raw", f), os.path.join(dest, "raw", f))


if __name__ == "__main__":
    main(sys.argv[1])
