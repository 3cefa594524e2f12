"""Code-generator plugin interface, mirroring
``pyrometheus/codegen/__init__.py:8-44`` (``CodeGenerationOptions`` and the
``CodeGenerator`` ABC with ``get_name`` / ``supports_overloading`` /
``generate``)."""

from abc import abstractmethod
from dataclasses import dataclass
from typing import Optional


@dataclass(frozen=True)
class CodeGenerationOptions:
    scalar_type: Optional[str] = None
    directive_offload: Optional[str] = None


class CodeGenerator:
    @staticmethod
    @abstractmethod
    def get_name() -> str:
        """Returns the name (slug) of the code generator."""

    @staticmethod
    @abstractmethod
    def supports_overloading() -> bool:
        """Returns whether the generated code supports operator overloading
        (array semantics)."""

    @staticmethod
    @abstractmethod
    def generate(name: str, sol, opts: CodeGenerationOptions = None) -> str:
        """Generate the thermochemistry code for the mechanism in *sol* (a
        Cantera ``Solution`` or :class:`pyrometheus_gb300.mechanism.Solution`)
        under the module/namespace *name*."""
