"""Copies the reference's example scene and deformation files (input data,
examples/*.json and examples/*.yaml of igrega348/xray_projection_render,
MIT licence) next to this script, so that the front-end tests can feed them
to XRayRenderer where the reference tree is absent.

    python tests/golden/examples/make_examples.py [reference root]

The files are copied byte for byte; nothing is generated.
"""
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
FILES = ["balls.json", "pillar_array.json", "cube_w_hole.yaml", "box_w_pped.yaml",
         "gyroid_example.yaml", "deformation_linear.yaml", "deformation_sigmoid.yaml"]


def main(ref_root):
    for name in FILES:
        shutil.copyfile(os.path.join(ref_root, "examples", name), os.path.join(HERE, name))
        print(name)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
