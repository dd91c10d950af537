"""The drop-in boundary: the engine library exports every entry point
that include/alis_c.h (the ALiS API) and include/alisgpu.h (the device
C-ABI) declare, and ALiS programs compile and link against it unchanged.
Loading the library does not touch a GPU; no compute is called here."""
import ctypes
import glob
import os
import re
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")


def declared_functions(header):
    text = open(os.path.join(INC, header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"#ifdef __cplusplus.*?#endif", "", text, flags=re.S)
    text = re.sub(r"^\s*#.*$", "", text, flags=re.M)
    # drop struct / union / enum bodies so only top-level declarations remain
    while True:
        t2 = re.sub(r"\{[^{}]*\}", " ", text)
        if t2 == text:
            break
        text = t2
    names = set()
    # prototypes: "... name(args);" or "... (name)(args);"
    for m in re.finditer(r"([A-Za-z_][A-Za-z0-9_]*)\s*\)?\s*\([^;{}]*\)\s*;", text):
        before = text[max(0, m.start() - 40):m.start()]
        if re.search(r"typedef[^;]*$", before):
            continue
        names.add(m.group(1))
    # parenthesised names: "void (h5)(...);"
    for m in re.finditer(r"\(\s*([A-Za-z_][A-Za-z0-9_]*)\s*\)\s*\([^;{}]*\)\s*;", text):
        names.add(m.group(1))
    # function-typedef declarations: "shape Box, Ball;" "field Ex, Ey;" ...
    for m in re.finditer(r"^\s*(shape|field|waveform|projmap)\s+([^;]+);", text, flags=re.M):
        for n in m.group(2).split(","):
            names.add(n.strip())
    for kw in ("sizeof", "if", "while", "for", "return", "typedef", "void", "int", "float", "double", "char"):
        names.discard(kw)
    return sorted(n for n in names if n)


@pytest.fixture(scope="module")
def engine():
    from alis_gb300 import build
    return ctypes.CDLL(build.build_engine())


@pytest.mark.parametrize("header", ["alis_c.h", "alisgpu.h"])
def test_library_exports_declared_symbols(engine, header):
    names = declared_functions(header)
    assert len(names) > (150 if header == "alis_c.h" else 15)
    missing = [n for n in names if not hasattr(engine, n)]
    assert not missing, missing


def test_product_does_not_contain_oracle():
    from alis_gb300 import build
    so = build.build_engine()
    out = subprocess.run(["nm", "-D", "--defined-only", so], capture_output=True, text=True).stdout
    for sym in ("curlStep", "ff32X", "ff64X", "psiX"):
        assert sym not in out


def _examples():
    from alis_gb300 import build
    ref = build.reference_root()
    return sorted(glob.glob(os.path.join(ref, "examples", "*.c"))) if ref else []


EXAMPLES = _examples()


@pytest.mark.skipif(not EXAMPLES, reason="reference examples not present on this machine")
@pytest.mark.parametrize("example", EXAMPLES, ids=[os.path.basename(e) for e in EXAMPLES])
def test_reference_example_compiles_and_links(engine, example):
    """Each ALiS example program builds unchanged against the engine."""
    from alis_gb300 import build
    with tempfile.TemporaryDirectory() as d:
        build.link_program(example, os.path.join(d, "prog"), "engine")


def test_engine_library_resolves_its_own_symbols():
    """Every alis_* / alisgpu_* symbol the engine references is defined in it."""
    import subprocess
    from alis_gb300 import build
    so = build.build_engine()
    out = subprocess.run(["nm", "-D", "--undefined-only", so], capture_output=True, text=True).stdout
    missing = [l.split()[-1] for l in out.splitlines() if l.split() and l.split()[-1].startswith(("alis_", "alisgpu_"))]
    assert not missing, missing
