"""Copy TSEMLib's example meshes into this folder as test fixtures.

The reference's examples run on three AFEPack .mesh files:
  examples/poisson_mixBC/cube.mesh         the unit cube as 6 tetrahedra, faces marked
                                           1 (Dirichlet) and 2 (Neumann, z = 0)
  examples/laplaceEig/cube.mesh            the same cube with every boundary face marked 1
  examples/KohnSham-Helium/cube_atom.mesh  [-10, 10]^3 as 184 tetrahedra around an atom
They are data, read through mesh.read_afepack by tests/test_gpu_reference_meshes.py
and tests/test_afepack_mesh.py.
Run in a checkout that has the reference available:

    python tests/golden/make_reference_meshes.py /path/to/TSEMLib
"""
import os
import shutil
import sys

FILES = {"examples/poisson_mixBC/cube.mesh": "ref_poisson_cube.mesh",
         "examples/laplaceEig/cube.mesh": "ref_laplace_cube.mesh",
         "examples/KohnSham-Helium/cube_atom.mesh": "ref_helium_cube_atom.mesh"}


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: make_reference_meshes.py <path of the TSEMLib checkout>")
    here = os.path.dirname(os.path.abspath(__file__))
    for src, dst in FILES.items():
        shutil.copyfile(os.path.join(sys.argv[1], src), os.path.join(here, dst))
        print("wrote", os.path.join(here, dst))


if __name__ == "__main__":
    main()
