"""The C-ABI libraries load and export every symbol the public header
declares (no GPU needed: no compute is called)."""

import ctypes
import os
import re

import pytest

from conftest import ROOT

HEADER_DIR = os.path.join(ROOT, "include")


def declared(header):
    with open(os.path.join(HEADER_DIR, header)) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(?:int|int64_t)\s+(pyro_\w+)\s*\(",
                                 text)))


def test_header_parses():
    names = declared("pyrometheus_gb300.h")
    assert "pyro_net_production_rates" in names
    assert len(names) >= 9


def test_mechanism_library_exports_header_symbols():
    from pyrometheus_gb300 import synthetic
    from pyrometheus_gb300.codegen.cuda import (CudaCodeGenerator,
                                                build_shared_library)
    sol = synthetic.config1_mechanism()
    lib = build_shared_library(CudaCodeGenerator.generate("t", sol), "abi")
    so = ctypes.CDLL(lib)
    for name in declared("pyrometheus_gb300.h"):
        assert hasattr(so, name), name
    ns, nr, nf = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    assert so.pyro_mechanism_info(ctypes.byref(ns), ctypes.byref(nr),
                                  ctypes.byref(nf), None, None) == 0
    assert (ns.value, nr.value, nf.value) == (9, 24, 2)


def test_block_thomas_library_exports_header_symbols():
    from pyrometheus_gb300 import native
    so = ctypes.CDLL(native.build_block_thomas())
    for name in declared("pyro_block_thomas.h"):
        assert hasattr(so, name), name
    so.pyro_block_thomas_work_doubles.restype = ctypes.c_int64
    # factors, b' and pivots per row; for nv <= 16 also S | t per row
    assert so.pyro_block_thomas_work_doubles(10, 7) == 7 * (100 + 20 + 110)
    assert so.pyro_block_thomas_work_doubles(54, 7) == 7 * (54 * 54 + 108)


@pytest.mark.parametrize("header,builder", [
    ("pyro_batched_lu.h", "build_batched_lu"),
    ("pyro_reactor_step.h", "build_reactor_step")])
def test_integrator_libraries_export_header_symbols(header, builder):
    from pyrometheus_gb300 import native
    so = ctypes.CDLL(getattr(native, builder)())
    names = declared(header)
    assert names
    for name in names:
        assert hasattr(so, name), name


def test_batched_lu_argument_errors_without_launch():
    from pyrometheus_gb300 import native
    lib = native.batched_lu_lib()
    assert lib.pyro_batched_lu_factor(None, None, None, -1, 4, None,
                                      None) == 1
    assert lib.pyro_batched_lu_factor(None, None, None, 3, 65, None,
                                      None) == 1
    assert lib.pyro_batched_lu_factor(None, None, None, 0, 4, None,
                                      None) == 0
    assert lib.pyro_batched_lu_solve(1, 1, None, None, 4, 1, 1, 4, 1, 2, 4,
                                     None) == 1


def test_argument_errors_without_launch():
    """Argument checks happen before any CUDA call, so they run without a
    GPU: a negative size or a short leading dimension is rejected."""
    from pyrometheus_gb300 import synthetic
    from pyrometheus_gb300.codegen.cuda import (CudaCodeGenerator,
                                                build_shared_library)
    from pyrometheus_gb300.thermochemistry import load_library
    sol = synthetic.config1_mechanism()
    so = load_library(build_shared_library(
        CudaCodeGenerator.generate("t", sol), "abi"))
    assert so.pyro_net_production_rates(None, 0, None, 0, None, 0, None, 0,
                                        -1, None) == 1
    assert so.pyro_net_production_rates(None, 0, None, 0, None, 0, None, 0,
                                        0, None) == 0
    assert so.pyro_net_production_rates(1, 0, 1, 0, 1, 4, 1, 8, 8,
                                        None) == 1
    assert so.pyro_species_property(9, 1, 0, 1, 8, 8, None) == 1


def test_no_cpu_fallback():
    """Without a CUDA device the drop-in class refuses to run."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    from pyrometheus_gb300 import get_thermochem_class, synthetic
    cls = get_thermochem_class(synthetic.config1_mechanism())
    with pytest.raises(RuntimeError, match="CUDA"):
        cls()


def test_compile_class_like_reference():
    """``compile_class(name, source, sol)`` builds the generated source into
    the named class and keeps the source (``python.py:689-697``); a source
    generated for another mechanism is refused."""
    import pyrometheus_gb300 as pg
    from pyrometheus_gb300 import synthetic
    sol = synthetic.config1_mechanism()
    src = pg.generate("Thermochemistry", sol)
    cls = pg.compile_class("Thermochemistry", src, sol)
    assert cls.__name__ == "Thermochemistry"
    assert cls._MODULE_SOURCE_CODE == src
    with pytest.raises(ValueError, match="9 species"):
        pg.compile_class("Thermochemistry", src,
                         synthetic.config2_mechanism())


def test_generator_options_like_reference():
    from pyrometheus_gb300 import CodeGenerationOptions, synthetic
    from pyrometheus_gb300.codegen.cuda import CudaCodeGenerator
    sol = synthetic.config1_mechanism()
    with pytest.raises(TypeError):
        CudaCodeGenerator.generate(
            "t", sol, CodeGenerationOptions(directive_offload="acc"))
    with pytest.raises(TypeError):
        CudaCodeGenerator.generate(
            "t", sol, CodeGenerationOptions(scalar_type="float"))
    assert CudaCodeGenerator.get_name() == "cuda"
    assert CudaCodeGenerator.supports_overloading()


def test_scheduling_fences_are_opt_in():
    """``fence_every`` puts an empty memory-clobber ``asm`` after every k-th
    reaction of the unrolled body and nowhere by default."""
    from pyrometheus_gb300 import synthetic
    from pyrometheus_gb300.codegen.cuda import (CudaCodeGenerator,
                                                CudaGenerationOptions)
    sol = synthetic.config1_mechanism()
    fence = 'asm volatile("" ::: "memory");'
    assert fence not in CudaCodeGenerator.generate("t", sol)
    n_rx = len(sol.reactions())
    for k in (1, 4, 7):
        src = CudaCodeGenerator.generate(
            "t", sol, CudaGenerationOptions(fence_every=k))
        assert src.count(fence) == (n_rx - 1) // k
    with pytest.raises(ValueError, match="fence_every"):
        CudaCodeGenerator.generate("t", sol,
                                   CudaGenerationOptions(fence_every=0))


@pytest.mark.parametrize("n_reactions", [24, 56, 60, 64])
def test_jacobian_groups_fill_whole_warps(n_reactions):
    """The Jacobian kernel's state groups (8 lanes per state for small
    mechanisms) fill whole warps of the CTA, whatever the shared memory per
    state allows: 60 reactions on 9 species leave room for 45 states per
    CTA, which the generator rounds down to 44 (a half-filled warp would
    break the groups' warp-wide sums)."""
    from pyrometheus_gb300 import synthetic
    from pyrometheus_gb300.codegen.cuda import CudaCodeGenerator
    sol = synthetic.make_mechanism(synthetic.SPECIES_9, n_reactions, 6, 4, 2,
                                   seed=5, name="wide9",
                                   orient_temperature=1500.0)
    src = CudaCodeGenerator.generate("m", sol)
    g = {k: int(re.search(rf"#define {k} (\d+)", src).group(1))
         for k in ("JGROUP", "JGROUPS")}
    assert g["JGROUP"] == 8
    assert (g["JGROUP"] * g["JGROUPS"]) % 32 == 0
    assert g["JGROUP"] * g["JGROUPS"] <= 512


def _table(src, name):
    m = re.search(rf"{name}\[[^\]]*\](?:\[[^\]]*\])? = \{{([^}}]*)\}}", src)
    return [int(v, 0) for v in m.group(1).replace("\n", " ").split(",")
            if v.strip()]


@pytest.mark.parametrize("which", ["config1", "config2", "wide9", "mid18"])
def test_jacobian_lane_tables(which):
    """The generated tables of the Jacobian kernel: every reaction runs on
    exactly one (round, lane); with whole-warp groups each warp's block of
    a round holds one kind of reaction; the per-species parts cover each
    species' slot list exactly once, in order, the first part the owner,
    the owners' lists naming the other parts' scratch slots."""
    from pyrometheus_gb300 import synthetic
    from pyrometheus_gb300.codegen.cuda import CudaCodeGenerator, _Model
    sol = {"config1": synthetic.config1_mechanism,
           "config2": synthetic.config2_mechanism,
           "wide9": lambda: synthetic.make_mechanism(
               synthetic.SPECIES_9, 60, 6, 4, 2, seed=5, name="wide9",
               orient_temperature=1500.0),
           "mid18": lambda: synthetic.make_mechanism(
               list(synthetic.SPECIES_53[:17]) + ["N2"], 40, 5, 3, 1,
               seed=7, name="mid18", orient_temperature=1500.0)}[which]()
    src = CudaCodeGenerator.generate("m", sol)
    jg = int(re.search(r"#define JGROUP (\d+)", src).group(1))
    nr = sol.n_reactions
    lane_rx = _table(src, "jq_lane_rx")
    assert sorted(q for q in lane_rx if q >= 0) == list(range(nr))
    flags = _table(src, "jq_flags")
    if jg >= 32:
        for b0 in range(0, len(lane_rx), 32):
            kinds = {flags[q] & 3 for q in lane_rx[b0:b0 + 32] if q >= 0}
            assert len(kinds) <= 1
    m = _Model(sol)
    sp = _table(src, "jq_sp")
    si0 = _table(src, "jg_si0")
    si_slot = _table(src, "jg_si_slot")
    p_sp, p_s0, p_s1 = (_table(src, n) for n in ("jp_sp", "jp_s0", "jp_s1"))
    p_slot = _table(src, "jp_slot")
    x0, xslot = _table(src, "jp_x0"), _table(src, "jp_xslot")
    for k in range(m.S):
        parts = [e for e, s_ in enumerate(p_sp) if s_ == k]
        assert parts, k
        cover = [a for e in parts for a in range(p_s0[e], p_s1[e])]
        assert cover == list(range(si0[k], si0[k + 1]))
        assert all(sp[si_slot[a]] == k for a in cover)
        owners = [e for e in parts if p_slot[e] < 0]
        assert len(owners) == 1 and owners[0] == parts[0]
        assert sorted(xslot[x0[k]:x0[k + 1]]) == sorted(
            p_slot[e] for e in parts[1:])


def test_cli_writes_source(tmp_path):
    from pyrometheus_gb300 import synthetic
    from pyrometheus_gb300.cli import main
    from pyrometheus_gb300.yaml_mech import dump_mechanism
    mech = tmp_path / "m.yaml"
    mech.write_text(dump_mechanism(synthetic.config1_mechanism()))
    out = tmp_path / "m.cu"
    main(["-l", "cuda", "-m", str(mech), "-o", str(out), "-n", "m"])
    src = out.read_text()
    assert "#define NS 9" in src and '#include "kinetics.cuh"' in src
