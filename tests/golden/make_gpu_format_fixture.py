"""Write, on a GPU, the files this build's fluid3D stage produces, for the
CPU tests that read them with the reference's own readers.

Runs a 10x12x8 FP64 plume (column source, vorticity 1, the reference's walls
and stop test) for STEPS steps through the C ABI, appending the stream rows
after every step (plume_append_streams) and writing the last step's state
file (plume_write_state, gzip level 1).  Stores in <out>/: the state file,
the six streams' .transpose and .dims files, and fields.npz with every field
downloaded from the device after the last step.  The reference's readGz
(FLUID_3D_MIC.cpp:1115-1246) and svdOutOfCoreMultiple must then read these
files unchanged (tests/test_formats.py).

Usage (on a GPU): python tests/golden/make_gpu_format_fixture.py <out dir>
The committed copy is tests/golden/gpu_format_10x12x8/.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from cfs_plume_gb300 import _abi  # noqa: E402
from cfs_plume_gb300.plume import Plume  # noqa: E402

RES = (10, 12, 8)
STEPS = 4


def main():
    out = sys.argv[1] if len(sys.argv) > 1 else os.path.join(HERE, "gpu_format_10x12x8")
    out = out if out.endswith("/") else out + "/"
    os.makedirs(out, exist_ok=True)
    g = Plume(_abi.default_params(res=RES, vorticity_eps=1.0))
    for s in range(STEPS):
        g.add_source(s)
        g.step()
        g.append_streams(out)
    g.write_state(out + "fluid.%04d.fluid3d.gz" % (STEPS - 1))
    fields = {n: g.field(n) for n in _abi.FIELDS}
    np.savez_compressed(out + "fields.npz", res=np.array(RES), steps=STEPS, vorticity_eps=1.0, **fields)
    g.close()
    print("wrote", sorted(os.listdir(out)))


if __name__ == "__main__":
    main()
