"""Fixture of the reference's coarse vortex mesh: tests/golden/vortex_coarse_mesh.npz.

Reads tests/shallowWaterVortex/shallowWaterVortex_20x10cells.msh of an oceano
checkout (directory given by the environment variable OCEANO_REFERENCE) and
stores its 200 quadrilaterals (4 vertices each) and the tagged boundary lines
(curve entity, its physical tag = boundary id, 2 vertices).  Run from the repository root:

    OCEANO_REFERENCE=<oceano checkout> python tests/golden/make_mesh_fixture.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
MSH = os.path.join("tests", "shallowWaterVortex", "shallowWaterVortex_20x10cells.msh")
OUT = os.path.join(HERE, "vortex_coarse_mesh.npz")


def read_msh4(path):
    """Quads, tagged lines and the physical tag of every curve entity of a Gmsh
    4.1 ASCII file."""
    lines = open(path).read().split("\n")
    i = lines.index("$Entities")
    n_pts, n_curves = map(int, lines[i + 1].split()[:2])
    curve_tag = {}
    for j in range(n_curves):
        f = lines[i + 2 + n_pts + j].split()
        n_phys = int(f[7])
        curve_tag[int(f[0])] = int(f[8]) if n_phys else -1
    i = lines.index("$Nodes")
    nb, _ = map(int, lines[i + 1].split()[:2])
    coords = {}
    k = i + 2
    for _ in range(nb):
        _, _, _, cnt = map(int, lines[k].split())
        tags = [int(lines[k + 1 + j]) for j in range(cnt)]
        for j in range(cnt):
            coords[tags[j]] = tuple(map(float, lines[k + 1 + cnt + j].split()))
        k += 1 + 2 * cnt
    i = lines.index("$Elements")
    nb = int(lines[i + 1].split()[0])
    k = i + 2
    quads, tagged = [], []
    for _ in range(nb):
        _, ent, etype, cnt = map(int, lines[k].split())
        for j in range(cnt):
            f = list(map(int, lines[k + 1 + j].split()))
            if etype == 3:
                quads.append([coords[n][:2] for n in f[1:]])
            elif etype == 1:
                tagged.append((ent, [coords[n][:2] for n in f[1:]]))
        k += 1 + cnt
    return quads, tagged, curve_tag


def main():
    root = os.environ.get("OCEANO_REFERENCE")
    if not root:
        sys.exit("set OCEANO_REFERENCE to an oceano checkout")
    quads, tagged, curve_tag = read_msh4(os.path.join(root, MSH))
    np.savez(OUT, quads=np.asarray(quads, np.float64),
             line_entity=np.asarray([t[0] for t in tagged], np.int32),
             line_physical=np.asarray([curve_tag[t[0]] for t in tagged], np.int32),
             lines=np.asarray([t[1] for t in tagged], np.float64))
    print(OUT, len(quads), "quads", len(tagged), "lines")


if __name__ == "__main__":
    main()
