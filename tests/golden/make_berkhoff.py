"""Write tests/golden/berkhoff.npz from the reference's Berkhoff (1982) shoal
benchmark (benchmarks/car_berkhoff_2d in the reference repository):

  params      the deck's hot-path keys, parsed from work/input.txt by this
              package's read_input_txt, as JSON text
  depth_um    input/depth.txt (DepthFormat = ELE: Mglob x Nglob cell depths,
              one row of 600 values per J) in integer micrometres, which
              holds the file's six decimals exactly
  height_ref  postprocessing/height_full.dat: the wave height the reference
              computed with postprocessing/calcheight.m (mean over the last
              five wave periods of the crest-to-trough range of the eta
              files), 600 x 200, float32 (the file prints 8 digits)
  sec1..sec5  the laboratory transects across the shoal, section*.dat
              (y in m, wave amplitude in mm); sec678 the three
              alongshore-parallel transects (x in m, three amplitudes)

The GPU tests cannot read the reference at run time, so this fixture
carries what they need.  Run here, where the reference is mounted:
    python tests/golden/make_berkhoff.py /path/to/reference
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))


def main(ref):
    import __graft_entry__
    fw = __graft_entry__.load_package()
    base = os.path.join(ref, "benchmarks", "car_berkhoff_2d")
    deck = fw.read_input_txt(os.path.join(base, "work", "input.txt"))
    keep = {k: v for k, v in deck.items() if k in fw.PARAM_DEFAULTS or k in ("SPONGE_ON", "CONSTRUCTION")}
    M, N = int(deck["Mglob"]), int(deck["Nglob"])
    rows = [np.array(line.split(), dtype=float)
            for line in open(os.path.join(base, "input", "depth.txt")) if line.strip()]
    depth = np.array(rows).T            # (M, N): row J of the file holds I = 1..M
    assert depth.shape == (M, N), depth.shape
    depth_um = np.rint(depth * 1e6).astype(np.int32)
    assert np.array_equal(depth_um / 1e6, depth)
    height = np.loadtxt(os.path.join(base, "postprocessing", "height_full.dat"))
    assert height.shape == (M, N), height.shape
    out = {"params": np.array(json.dumps(keep)), "depth_um": depth_um, "height_ref": height.astype(np.float32)}
    for k in range(1, 6):
        out["sec%d" % k] = np.loadtxt(os.path.join(base, "postprocessing", "section%d.dat" % k))
    out["sec678"] = np.loadtxt(os.path.join(base, "postprocessing", "section678.dat"))
    np.savez_compressed(os.path.join(HERE, "berkhoff.npz"), **out)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
