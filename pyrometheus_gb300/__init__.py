"""pyrometheus_gb300: GB300 (sm_103a) code generation for pyrometheus'
per-state thermochemistry and kinetics.

The package mirrors ``pyrometheus/__init__.py:40-52``: a registry of code
generators keyed by name (here the ``cuda`` target) and the default
generator's static methods exposed as module functions (``generate``,
``build_module``, ``get_thermochem_class``).
"""

import typing

from .codegen import CodeGenerator, CodeGenerationOptions  # noqa: F401
from .codegen.cuda import CudaCodeGenerator, CudaGenerationOptions  # noqa

__version__ = "0.1.0"


def get_code_generators() -> typing.Dict[str, CodeGenerator]:
    return {CudaCodeGenerator.get_name(): CudaCodeGenerator}


# The CUDA generator is the default one: expose its static methods as
# module-level functions, as the reference does for its Python generator.
for _name, _method in CudaCodeGenerator.__dict__.items():
    if isinstance(_method, staticmethod):
        globals()[_name] = getattr(CudaCodeGenerator, _name)
del _name, _method
