"""Times the PIC++ reference (compiled from its own sources by the Makefile
in the parent directory) and the oracle on the same explicit Buneman/Yee
sample -- 16^3 cells, 16 particles per cell and species, two species, one
host core each -- to show how fast the oracle, which stands in for the
reference on machines without its sources, runs against the reference
itself.  The harness reports the wall time of its step loop alone.

    PICPP_REFERENCE_SRC=<PIC++ source directory> python oracle/ref/time_against_oracle.py [steps]
"""
import os
import struct
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import pyoracle as O  # noqa: E402
from picpp_gb300 import initstate as I  # noqa: E402


def main():
    steps = int(sys.argv[1]) if len(sys.argv) > 1 else 40
    st = I.buneman_plasma(16, 16, 16, ppc=16, seed=11)
    box = st.box
    npart = sum(len(s["cell"]) for s in st.species)
    exe = O.build_reference()
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        with open(fin, "wb") as f:
            f.write(struct.pack("<10i", 0, box.nx, box.ny, box.nz, len(st.species), steps, 0, 0, 0, 0))
            f.write(struct.pack("<11d", box.dx, box.dt, box.theta, box.eta, 0.5, 0, 0, 0, 0, 0, 0))
            for sp in st.species:
                x, y, z = I.positions(box, sp)
                f.write(struct.pack("<3dq", sp["q"], sp["m"], sp["w"], len(sp["cell"])))
                for a in (x, y, z, sp["px"], sp["py"], sp["pz"]):
                    f.write(np.ascontiguousarray(a, dtype="<f8").tobytes())
            f.write(np.ascontiguousarray(st.E, dtype="<f8").tobytes())
            f.write(np.ascontiguousarray(st.B, dtype="<f8").tobytes())
        out = subprocess.run([exe, fin, fout], capture_output=True, text=True, check=True).stdout
    t_ref = float(out.split("steps in")[1].split()[0])
    g = O.make_grid(box)
    E, B = st.E.copy(), st.B.copy()
    t0 = time.perf_counter()
    for _ in range(steps):
        O.buneman_step(g, st.species, E, B)
    t_orc = time.perf_counter() - t0
    print(f"{npart} particles, {steps} steps: reference {npart * steps / t_ref:.3e} particle-steps/s, "
          f"oracle {npart * steps / t_orc:.3e} particle-steps/s (oracle / reference {t_ref / t_orc:.2f})")


if __name__ == "__main__":
    main()
