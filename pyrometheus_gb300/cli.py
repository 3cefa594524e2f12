"""Command line, mirroring ``pyrometheus/cli.py:11-42``:

    python -m pyrometheus_gb300 -l cuda -m mech.yaml -o out.cu -n NAME [-p PHASE]

writes the generated CUDA translation unit; ``--build`` also compiles it to a
shared library next to the output (``out.so``).
"""

import argparse

from . import get_code_generators, __version__
from .yaml_mech import load_mechanism


def main(argv=None):
    generators = get_code_generators()
    parser = argparse.ArgumentParser(
        prog="pyrometheus_gb300",
        description="Code generation for combustion thermochemistry "
                    "(GB300 CUDA target).")
    parser.add_argument("--version", action="version",
                        version=f"%(prog)s {__version__}")
    parser.add_argument("-l", "--lang", "--language",
                        help="Language to generate code for.",
                        choices=generators.keys(), required=True)
    parser.add_argument("-m", "--mech", "--mechanism",
                        help="Path to the mechanism file.", required=True)
    parser.add_argument("-o", "--output", help="Path to the output file.",
                        required=True)
    parser.add_argument("-n", "--name", "--namespace",
                        help="Namespace to use for the generated code.",
                        required=True)
    parser.add_argument("-p", "--phase",
                        help="Phase name to use for the generated code.")
    parser.add_argument("--build", action="store_true",
                        help="Also compile the output to a shared library.")
    args = parser.parse_args(argv)

    gen = generators[args.lang]
    source = gen.generate(args.name, load_mechanism(args.mech, args.phase))
    with open(args.output, "w") as f:
        f.write(source)
    if args.build:
        import os
        import shutil
        lib = gen.build_module(source, args.name)
        dst = os.path.splitext(args.output)[0] + ".so"
        shutil.copyfile(lib, dst)
