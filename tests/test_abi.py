"""The C-ABI library builds, loads without a GPU and exports every entry point
declared in include/mpcmd.h; the config struct layouts agree (CPU only: no
compute calls)."""
import ctypes as C
import os
import re
import subprocess

from conftest import ROOT
import main_gb300
from main_gb300 import config
from oracle import oracle as O

HEADER = os.path.join(ROOT, "include", "mpcmd.h")


def declared_functions():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[\w]+\s*\*?\s*(mpcmd_\w+)\s*\(", src, re.M)))


def test_library_exports_every_declared_function():
    lib = main_gb300.lib()
    names = declared_functions()
    assert len(names) >= 30
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(main_gb300.SIGNATURES), set(names) ^ set(main_gb300.SIGNATURES)


def test_contract_rng_is_shared_with_the_oracle():
    for args in [(1, 1, 0, 0, 50, 0), (1, 2, 123, 0, 100, 1), (2 ** 63 + 5, 4, 99999, 7, 12345, 0)]:
        assert main_gb300.contract_u01(*args) == O.contract_u01(*args)


def test_error_strings():
    lib = main_gb300.lib()
    for code in range(11):
        assert lib.mpcmd_error_string(code)


def test_config_layout_matches_header_and_oracle():
    # compile a probe of the real header with gcc and compare field offsets
    import tempfile
    probe = tempfile.mkdtemp(prefix="mpcmd_layout_")
    src = os.path.join(probe, "layout_probe.c")
    exe = os.path.join(probe, "layout_probe")
    fields = [f for f, _ in config.FIELDS]
    with open(src, "w") as f:
        f.write('#include <stdio.h>\n#include <stddef.h>\n#include "mpcmd.h"\n#include "oracle.h"\nint main(void){\n')
        f.write('printf("%zu %zu\\n", sizeof(mpcmd_config), sizeof(orc_params));\n')
        for name in fields:
            f.write('printf("%%zu\\n", offsetof(mpcmd_config, %s));\n' % name)
        for name, _ in O.PARAM_FIELDS:
            f.write('printf("%%zu\\n", offsetof(orc_params, %s));\n' % name)
        f.write("return 0;}\n")
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "oracle"), "-o", exe, src],
                   check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split()
    size_c, size_o = int(out[0]), int(out[1])
    offs = [int(v) for v in out[2:]]
    assert size_c == C.sizeof(config.MpcmdConfig)
    assert size_o == C.sizeof(O.OrcParams)
    for i, name in enumerate(fields):
        assert offs[i] == getattr(config.MpcmdConfig, name).offset, name
    for j, (name, _) in enumerate(O.PARAM_FIELDS):
        assert offs[len(fields) + j] == getattr(O.OrcParams, name).offset, name
        # the two structs share their layout; the oracle's engine_only words
        # sit where the engine config holds precision and shell_capacity
        twin = "precision" if name == "engine_only" else name
        assert getattr(O.OrcParams, name).offset == getattr(config.MpcmdConfig, twin).offset, name
    assert C.sizeof(O.OrcParams) == C.sizeof(config.MpcmdConfig)


def test_reference_decks_parse():
    from conftest import reference_root
    ref = reference_root()
    if ref is None:
        import pytest
        pytest.skip("MPCMD_REFERENCE_ROOT does not name a reference checkout")
    d = config.read_collective_input(os.path.join(ref, "collective_code", "input.txt"))
    c = config.collective_config(d)
    assert (c["lx"], c["ly"], c["lz"], c["n_dimers"]) == (64, 64, 32, 20)
    assert c["mpc_every"] == 20 and c["sort_every"] == 10000
    s = config.read_selkov_input(os.path.join(ref, "selkov_code", "Input_SelkovDimer.txt"))
    k = config.selkov_config(s)
    assert k["n_solvent"] == 230400 + 54400 + 422400
    assert abs(k["kT"] - 0.2) < 1e-15
