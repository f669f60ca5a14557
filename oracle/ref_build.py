"""Recipe for ``oracle/_ref``: the reference's own kernels as a CPU baseline.

TEST/BASELINE INFRASTRUCTURE ONLY (used by ``bench.py --impl reference`` and
the CPU-baseline leg; never by the product).

Where the reference source is available, ``build()`` dumps the C++ that the
reference translator generates for ``LifelikeCA`` (its interactive-rule Life
model, ``examples/game_of_life.py:183-203``) at every lattice size of the
ensemble benchmark -- its kernels bake the size in as ``#define``s -- into
``oracle/_ref/ref_lifelike_<w>x<h>.cpp`` and compiles each with g++/OpenMP
(``ref_harness.compile_cpp``).  Without the reference (the GPU machine) it only
compiles the ``.cpp`` files that are already there.
"""
import glob
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
SIDES = (64, 128, 256, 512, 1024)


def reference_root(required=False):
    """The reference checkout: ``$XK_REFERENCE_SRC``, else a checkout named
    ``reference`` beside this repository.  Returns None when neither holds
    the ``xentica`` package, or exits with a message when ``required``."""
    env = os.environ.get("XK_REFERENCE_SRC")
    beside = os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")
    for root in ([env] if env else []) + [beside]:
        if os.path.isdir(os.path.join(root, "xentica")):
            return os.path.abspath(root)
    if required:
        raise SystemExit("reference checkout not found: set XK_REFERENCE_SRC to the directory "
                         "holding the xentica package (tried %s)"
                         % ", ".join(([env] if env else []) + [beside]))
    return None


def _generate(ref_root):
    from ref_harness import run_reference
    manifest = {}
    for w in SIDES:
        for h in SIDES:
            name = "lifelike_%dx%d" % (w, h)
            cpp = os.path.join(REF_DIR, "ref_%s.cpp" % name)
            if not os.path.exists(cpp):
                run_reference({"model": "examples.game_of_life:LifelikeCA",
                               "experiment": "examples.game_of_life:GOLExperiment2",
                               "exp_overrides": {"size": [w, h]}, "checkpoints": [],
                               "workdir": REF_DIR, "name": name, "threads": 1}, ref_root)
            manifest[name] = {"model": "LifelikeCA", "width": w, "height": h,
                              "cpp": os.path.basename(cpp), "so": "ref_%s.so" % name}
    with open(os.path.join(REF_DIR, "manifest.json"), "w") as fh:
        json.dump(manifest, fh, indent=1)


def build():
    """Generate (when the reference is present) and compile the baseline."""
    os.makedirs(REF_DIR, exist_ok=True)
    sys.path.insert(0, HERE)
    from ref_harness import compile_cpp
    root = reference_root()
    if root:
        _generate(root)
    for cpp in sorted(glob.glob(os.path.join(REF_DIR, "ref_lifelike_*.cpp"))):
        so = cpp[:-4] + ".so"
        if not os.path.exists(so) or os.path.getmtime(so) < os.path.getmtime(cpp):
            compile_cpp(cpp, so)
    return REF_DIR


def available():
    """Manifest of compiled reference kernels, or None."""
    path = os.path.join(REF_DIR, "manifest.json")
    if not os.path.exists(path):
        return None
    with open(path) as fh:
        manifest = json.load(fh)
    for entry in manifest.values():
        if not os.path.exists(os.path.join(REF_DIR, entry["so"])):
            return None
    return manifest


if __name__ == "__main__":
    print(build())
