"""Writes tests/golden/mesh_seeds.npz from the reference's mesh seed files.

    python tests/golden/make_mesh_seeds.py <lpm>/mesh_seeds

The reference builds every uniform mesh from a seed file read by
MeshSeed::read_file (src/mesh/lpm_mesh_seed.cpp:20-201): line 1 is a header,
the next nverts + nfaces lines hold the vertex coordinates followed by the
face centres, then edge (origin, destination, left face, right face), face
vertex and face edge tables follow their header lines ("edgeO", "faceverts",
"faceedges").  This script parses the three seeds on the direct-sum path
(icosahedral triangles, cubed sphere, unit square) the same way and stores
them as arrays, so the oracle's mesh restatement and the tests take their
seed from the reference's own numbers without reading the reference at run
time.  Python's float() rounds decimal text to the nearest double, as the
reference's istream extraction does.
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent

# name: (file, ndim, nverts, nfaces, nedges, vertices per face); the counts
# are IcosTriSphereSeed / CubedSphereSeed / QuadRectSeed's (src/mesh/lpm_mesh_seed.hpp)
SEEDS = {
    "icos": ("icosTriSphereSeed.dat", 3, 12, 20, 30, 3),
    "cubed": ("cubedSphereSeed.dat", 3, 8, 6, 12, 4),
    "quad": ("quadRectSeed.dat", 2, 9, 4, 12, 4),
}


def parse(path: Path, ndim: int, nverts: int, nfaces: int, nedges: int, nfv: int):
    lines = path.read_text().splitlines()
    ncrds = nverts + nfaces
    crds = np.array([[float(t) for t in lines[1 + i].split()[:ndim]] for i in range(ncrds)])

    def table(key: str, n: int, width: int) -> np.ndarray:
        h = next(i for i, line in enumerate(lines) if key in line)
        return np.array([[int(t) for t in lines[h + 1 + i].split()[:width]] for i in range(n)],
                        dtype=np.int64)

    return crds, table("edgeO", nedges, 4), table("faceverts", nfaces, nfv), \
        table("faceedges", nfaces, nfv)


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: make_mesh_seeds.py <directory holding the reference's mesh seed files>")
    seed_dir = Path(sys.argv[1])
    out = {}
    for name, (fname, ndim, nv, nf, ne, nfv) in SEEDS.items():
        crds, edges, fverts, fedges = parse(seed_dir / fname, ndim, nv, nf, ne, nfv)
        out[f"{name}_crds"] = crds
        out[f"{name}_edges"] = edges
        out[f"{name}_faceverts"] = fverts
        out[f"{name}_faceedges"] = fedges
    np.savez_compressed(HERE / "mesh_seeds.npz", **out)
    print("wrote", HERE / "mesh_seeds.npz")


if __name__ == "__main__":
    main()
