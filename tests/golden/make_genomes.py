"""Writes the benchmark workloads' genomes to tests/golden/genomes/ as flam3 XML.

The genomes are the library's seeded synthetic genomes (rf_flame_synthesize, drawn with
std::mt19937_64 in a documented order), serialised once so that the CPU reference arm of
bench.py and the tests read the very same genome without loading the CUDA library:

  small.flam3          3 xforms (seed 0), 512x512 bins           (plain chaos game, small)
  frame1080.flam3      8 xforms + final (seed 1), julian/ngon/pdj forced, 3840x2160 bins
                       (the 1080p frame at supersample 2; camera: [-2.5, 2.5] spans the height)
  contract.flam3       6 contracting xforms (seed 4), 1920x1080 bins
  spacefill.flam3      16 spherical+swirl xforms (seed 5), 8192x8192 bins
  batch_frame0.flam3   frame 0 of the batched animation: seed 2 (4 xforms) interpolated towards
                       seed 3 (10 xforms) at t = 0, 1024x768 bins

and, when the reference checkout is present, a copy of its one real genome
(flames/electricsheep.247.11256.flam3: 10 xforms with a post affine, a final xform, a rotated
camera) as electricsheep.247.11256.flam3.

Usage: python tests/golden/make_genomes.py [reference_dir]
The reference directory defaults to $REFRAKT_REFERENCE, else <repo>/../reference; without a
checkout there the copy is skipped.
"""
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "genomes")

# name: (kind, seed, bins_w, bins_h, n_xforms, final_xform, force_parametric)
SYNTHETIC = {
    "small": (0, 0, 512, 512, 0, False, False),
    "frame1080": (1, 1, 3840, 2160, 8, True, True),
    "contract": (2, 4, 1920, 1080, 0, False, False),
    "spacefill": (3, 5, 8192, 8192, 0, False, False),
}
REFERENCE_GENOME = "electricsheep.247.11256.flam3"


def synthesize_all(R, comp):
    """name -> flam3 XML of every workload genome (the product's synthesiser)."""
    out = {}
    for name, (kind, seed, w, h, nx, fin, forced) in SYNTHETIC.items():
        f = R.Flame.synthesize(comp, kind, seed, w, h, n_xforms=nx, final_xform=fin, force_parametric=forced)
        out[name] = f.to_xml()
    a = R.Flame.synthesize(comp, R.SYNTH_RANDOM, 2, 1024, 768, n_xforms=4)
    b = R.Flame.synthesize(comp, R.SYNTH_RANDOM, 3, 1024, 768, n_xforms=10)
    out["batch_frame0"] = a.interpolate(b, 0.0).to_xml()
    return out


def main():
    sys.path.insert(0, ROOT)
    import refrakt_gb300 as R
    R.build()
    comp = R.FlameCompiler()
    os.makedirs(OUT, exist_ok=True)
    for name, xml in synthesize_all(R, comp).items():
        with open(os.path.join(OUT, name + ".flam3"), "w") as f:
            f.write(xml)
    ref = sys.argv[1] if len(sys.argv) > 1 else os.path.normpath(
        os.environ.get("REFRAKT_REFERENCE") or os.path.join(ROOT, os.pardir, "reference"))
    if os.path.isfile(os.path.join(ref, "flames", REFERENCE_GENOME)):
        shutil.copyfile(os.path.join(ref, "flames", REFERENCE_GENOME), os.path.join(OUT, REFERENCE_GENOME))
    print(sorted(os.listdir(OUT)))


if __name__ == "__main__":
    main()
