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
        description="Generate thermochemistry code for a mechanism; the "
                    "cuda target emits a GB300 (sm_103a) translation "
                    "unit.")
    parser.add_argument("--version", action="version",
                        version=f"%(prog)s {__version__}")
    parser.add_argument("-l", "--lang", "--language",
                        help="target language of the generated code",
                        choices=generators.keys(), required=True)
    parser.add_argument("-m", "--mech", "--mechanism",
                        help="mechanism file (Cantera YAML)", required=True)
    parser.add_argument("-o", "--output", help="file to write the generated code to",
                        required=True)
    parser.add_argument("-n", "--name", "--namespace",
                        help="name of the generated class or namespace",
                        required=True)
    parser.add_argument("-p", "--phase",
                        help="phase of the mechanism file to read")
    parser.add_argument("--build", action="store_true",
                        help="also compile the output into a shared library")
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
