"""Regenerate the example-scene fixtures from the reference tree.

Copies the STL meshes of fogleman/fauxgl's examples (bowser.stl, hello.stl,
sphere.stl, cube.stl) gzipped into tests/golden/examples/, renders every
scene of tests/example_scenes.py on the oracle and writes the expected
RasterizeInfo and the sha256 digests of colour, depth and winner ids to
tests/golden/examples.json. The digests pin the oracle across machines (the
GPU test re-renders the oracle where it runs and checks both against them).

    python tests/golden/make_examples.py [reference tree, default /root/reference]
"""
import gzip
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def main():
    ref_root = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    from tests import example_scenes as E
    os.makedirs(E.EXAMPLES, exist_ok=True)
    for stl in ("bowser", "hello", "sphere", "cube"):
        with open(os.path.join(ref_root, "examples", stl + ".stl"), "rb") as f:
            data = f.read()
        with gzip.GzipFile(os.path.join(E.EXAMPLES, stl + ".stl.gz"), "wb", mtime=0) as g:
            g.write(data)
    out = {}
    for name in E.NAMES:
        ref, infos, mesh = E.render_oracle(name)
        out[name] = {"width": ref.width, "height": ref.height, "triangles": mesh.ntri,
                     "infos": [list(i) for i in infos],
                     **E.digests(ref.color(), ref.depth(), ref.winner())}
        print(name, out[name]["infos"], flush=True)
    with open(os.path.join(HERE, "examples.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
        f.write("\n")


if __name__ == "__main__":
    main()
