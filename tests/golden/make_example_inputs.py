"""Copies the reference's example inputs into tests/golden/example_problems/.

The reference (CaitlinChalk/Stress-Particle-SPH) ships no expected outputs, only the input
sets of its three example problems: the Drucker-Prager soil failure
(example_problems/soil_failure_bui_et_al_2008: inside approach SP1-3, standard SPH, outside
approach, velocity-vector update), the strain-localisation sample
(example_problems/strain_localisation_in_soil_sample: root, standard, SP1-3) and the
vertical cut (example_problems/vertical_slope: root, standard, SP1-3).  Each set is an
input.txt with a <name>.dat and a <name>.pts.  This script copies those three files of every
set, unchanged, so that the tests can run the sets on machines without the reference
checkout.  It only reads the reference; run it from the repository root:

    python tests/golden/make_example_inputs.py [path/to/reference]
"""
import glob
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "example_problems")


def main(ref):
    src = os.path.join(ref, "example_problems")
    sets = sorted(os.path.dirname(p) for p in glob.glob(src + "/**/input.txt", recursive=True)
                  if glob.glob(os.path.join(os.path.dirname(p), "*.dat")))
    n = 0
    for d in sets:
        rel = os.path.relpath(d, src)
        dst = os.path.join(OUT, rel)
        os.makedirs(dst, exist_ok=True)
        for f in ["input.txt"] + [os.path.basename(x) for x in glob.glob(d + "/*.dat")] + \
                 [os.path.basename(x) for x in glob.glob(d + "/*.pts")]:
            shutil.copyfile(os.path.join(d, f), os.path.join(dst, f))
            n += 1
    print("%d input sets, %d files -> %s" % (len(sets), n, OUT))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
