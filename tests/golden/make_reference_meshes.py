"""Copy the reference's own test meshes into this directory as fixtures.

NiHu's pulsating-sphere test reads OFF meshes of the unit sphere
(nihu/test/stallone_unit/helmholtz_3d_pulsating_sphere_test.cpp:40):
sphere_1_3.off (218 nodes, 432 flat triangles) and sphere_1_5.off (600 flat
quads).  This script copies them unchanged (they are data, read by
nihu_gb300.meshes.read_off), after checking that each parses as an OFF
mesh with the expected element count.  Run it where the reference tree is
present:

    python tests/golden/make_reference_meshes.py /root/reference
"""
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
FILES = {"sphere_1_3.off": 432, "sphere_1_5.off": 600}


def main(ref_root):
    sys.path.insert(0, os.path.join(HERE, "..", ".."))
    from nihu_gb300 import meshes
    for name, count in FILES.items():
        src = os.path.join(ref_root, "nihu", "test", "stallone_unit", name)
        nodes, elems = meshes.read_off(src)
        if len(elems) != count:
            raise SystemExit("%s: %d elements, expected %d" % (src, len(elems), count))
        shutil.copyfile(src, os.path.join(HERE, name))
        print("%s: %d nodes, %d elements" % (name, len(nodes), len(elems)))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
