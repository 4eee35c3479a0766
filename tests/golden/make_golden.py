"""Regenerate the golden fixtures of this directory from the reference's own data.

Reads (only in the development container, where the reference tree is mounted):
  pes/EMT-HAu.pes, pes/EMT-HPt.pes          -> emt_params.json (parsed parameter blocks)
  conf/latt/mxt_00000001.dat                 -> mxt_latt.npz (decoded geometry)
  example/md/RuNNer_input/{input.nn,scaling.data,weights.006.data}
  conf/example.POSCAR, conf/cart.POSCAR       -> poscar_ref.json (file text and its coordinate
                                               block parsed by numpy, independently of io)
  example/md/conf/latt/mxt_00000001.dat      -> runner_cgraphene.npz (parsed network +
                                               geometry) and runner_cgraphene_ref.npz
                                               (the oracle's own energy/forces/descriptors/
                                               neighbours: a regression fixture that keeps
                                               the oracle and the GPU path from drifting,
                                               not an independent golden vector)
Usage:  python tests/golden/make_golden.py <reference checkout>
        (default: MDT_REFERENCE_ROOT, else a directory named reference beside the repository)
"""
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

from md_tian2_gb300 import io, nene  # noqa: E402
from md_tian2_gb300 import constants as C  # noqa: E402


def main(ref):
    ref = Path(ref)
    out = {}
    for name, names in (("EMT-HAu.pes", ["H", "Au"]), ("EMT-HPt.pes", ["H", "Pt"])):
        p = io.read_pes(ref / "pes" / name, names, [True, False])
        out[name] = {k: p.values[k].tolist() for k in io.EMT_KEYS}
    (HERE / "emt_params.json").write_text(json.dumps(out, indent=1))

    u = io.read_mxt(ref / "conf" / "latt" / "mxt_00000001.dat")
    np.savez(HERE / "mxt_latt.npz", r=u.r, v=u.v, simbox=u.simbox, idx=u.idx, is_fixed=u.is_fixed,
             names=np.array(u.names), is_proj=u.is_proj)

    pos = {}
    for name in ("example.POSCAR", "cart.POSCAR"):
        text = (ref / "conf" / name).read_text()
        lines = text.splitlines()
        scale = float(lines[1].split()[0])
        cell = np.array([[float(x) for x in l.split()[:3]] for l in lines[2:5]])
        coords = np.array([[float(x) for x in l.split()[:3]] for l in lines[8:] if l.strip()])
        pos[name] = {"text": text, "scale": scale, "cell_rows": cell.tolist(), "coords": coords.tolist(),
                     "elements": lines[5].split()}
    (HERE / "poscar_ref.json").write_text(json.dumps(pos, indent=1))

    m = nene.read_runner(ref / "example" / "md" / "RuNNer_input")
    nene.save_npz(m, HERE / "runner_cgraphene.npz")
    g = io.read_mxt(ref / "example" / "md" / "conf" / "latt" / "mxt_00000001.dat")
    np.savez(HERE / "cgraphene_geometry.npz", r=g.r[:, 0, :], simbox=g.simbox)

    from oracle.oracle import NNOracle
    o = NNOracle(m)
    E, F, G, ea = o.energy_force(np.zeros(g.natoms, int), g.r[:, 0, :], g.simbox, want_G=True)
    x = g.r[:, 0, :] * C.ANG2BOHR
    lat = g.simbox.T * C.ANG2BOHR
    counts, nj, nn, nr = NNOracle.neighbors(x, lat, m.maxcut)
    np.savez(HERE / "runner_cgraphene_ref.npz", energy=E, forces=F, G=G, eatom=ea, nb_counts=counts, nb_j=nj,
             nb_n=nn)
    print("golden fixtures written")


if __name__ == "__main__":
    if len(sys.argv) > 1:
        main(sys.argv[1])
    else:
        sys.path.insert(0, str(HERE.parent.parent))
        from tests.refroot import reference_root
        root = reference_root()
        if root is None:
            sys.exit("no reference checkout: pass its path or set MDT_REFERENCE_ROOT")
        main(str(root))
