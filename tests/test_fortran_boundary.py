"""The Fortran side of the drop-in boundary, checked without a Fortran compiler (none exists on
this image or on the GPU machine).

The 2DENSE driver would call the library through the ISO_C_BINDING module include/dense_gpu.f90,
in place of the four per-stage calls of source/utility/general_main.f90:26-31. Here:
  * the bind(C) derived type dense_config_t, parsed from the module's source, laid out by the C
    rules that bind(C) guarantees (c_int 4 bytes, c_double 8 bytes, each at its natural alignment,
    arrays contiguous), must give every field the offset that gcc gives the C struct of
    include/dense2d.h, and the same size;
  * every procedure the module binds (bind(C, name="...")) must be declared in the header and
    exported by libdense2d.so;
  * the listing in INTEGRATION.md must be the committed module;
  * on a GPU, a C program that makes the driver's calls in its order and with its argument
    passing (tests/fortran_order_driver.c: column-major host arrays with four ghost layers,
    dense_stage(irk) three times per step, dense_download) must leave the state bit for bit where
    the CPU oracle does (strict kernels).
"""
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT, interior

INCLUDE = os.path.join(ROOT, "include")
F90 = os.path.join(INCLUDE, "dense_gpu.f90")
HEADER = os.path.join(INCLUDE, "dense2d.h")

KINDS = {"integer(c_int)": (4, 4), "real(c_double)": (8, 8)}


def bind_c_fields(src: str):
    """[(name, kind, count)] of `type, bind(C) :: dense_config_t`, in declaration order."""
    m = re.search(r"type\s*,\s*bind\s*\(\s*C\s*\)\s*::\s*dense_config_t\s*\n(.*?)\n\s*end\s+type",
                  src, flags=re.S | re.I)
    assert m, "no bind(C) dense_config_t in the module"
    out = []
    for line in m.group(1).splitlines():
        line = line.split("!")[0].strip()
        if not line:
            continue
        kind, names = [t.strip() for t in line.split("::")]
        kind = kind.replace(" ", "").lower()
        assert kind in KINDS, kind
        for name in [n.strip() for n in names.split(",")]:
            mm = re.fullmatch(r"(\w+)(?:\((\d+)\))?", name)
            assert mm, name
            out.append((mm.group(1), kind, int(mm.group(2) or 1)))
    return out


def c_layout(fields):
    """Offsets and size of a C struct with these members (natural alignment, no packing)."""
    off, align_max, offsets = 0, 1, {}
    for name, kind, count in fields:
        size, align = KINDS[kind]
        off = (off + align - 1) // align * align
        offsets[name] = off
        off += size * count
        align_max = max(align_max, align)
    return offsets, (off + align_max - 1) // align_max * align_max


def test_bind_c_type_matches_the_header_layout(tmp_path):
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not found")
    fields = bind_c_fields(open(F90).read())
    expect, expect_size = c_layout(fields)
    lines = "\n".join(f'    printf("%s %zu\\n", "{n}", offsetof(dense_config_t, {n}));'
                      for n, _, _ in fields)
    prog = tmp_path / "layout.c"
    prog.write_text("#include <stddef.h>\n#include <stdio.h>\n#include \"dense2d.h\"\n"
                    "int main(void) {\n" + lines +
                    '\n    printf("sizeof %zu\\n", sizeof(dense_config_t));\n    return 0;\n}\n')
    exe = tmp_path / "layout"
    subprocess.run([gcc, "-std=c99", "-I", INCLUDE, "-o", str(exe), str(prog)], check=True)
    got = dict(l.split() for l in subprocess.run([str(exe)], check=True, capture_output=True,
                                                 text=True).stdout.splitlines())
    for name, _, _ in fields:
        assert int(got[name]) == expect[name], (name, got[name], expect[name])
    assert int(got["sizeof"]) == expect_size
    # and the module names every member of the C struct (none left out)
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    body = re.search(r"typedef struct dense_config_t \{(.*?)\} dense_config_t;", text, flags=re.S).group(1)
    c_names = re.findall(r"\b(\w+)\s*(?:\[\d+\])?\s*[,;]", body)
    assert c_names == [n for n, _, _ in fields]


def test_bound_procedures_are_declared_and_exported(dense):
    names = re.findall(r'bind\(\s*C\s*,\s*name\s*=\s*"(\w+)"\s*\)', open(F90).read())
    assert len(names) >= 10
    header = open(HEADER).read()
    lib = dense.load_library()
    for n in names:
        assert re.search(rf"\b{n}\s*\(", header), n
        assert hasattr(lib, n), n


def test_integration_listing_is_the_committed_module():
    doc = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    listing = re.search(r"```fortran\n(module dense_gpu\n.*?end module dense_gpu\n)```", doc, flags=re.S)
    assert listing
    src = open(F90).read()
    assert src[src.index("module dense_gpu\n"):] == listing.group(1)


@pytest.fixture(scope="module")
def driver_exe(dense, tmp_path_factory):
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not found")
    lib = dense.LIB_PATH
    exe = tmp_path_factory.mktemp("driver") / "fortran_order_driver"
    subprocess.run([gcc, "-std=c99", "-O2", "-I", INCLUDE, "-o", str(exe),
                    os.path.join(ROOT, "tests", "fortran_order_driver.c"), lib,
                    "-Wl,-rpath," + os.path.dirname(lib)], check=True)
    return exe


@pytest.mark.gpu
@pytest.mark.parametrize("bench,split,recon,ni,nj", [
    (5, 105, 0, 96, 24),     # double Mach reflection, AdaWENO (reads the cell-centre rows)
    (11, 101, 253, 48, 40),  # periodic vortex, LLF + WENO-JS5
    (13, 104, 0, 32, 96),    # Rayleigh-Taylor, reflective sides, body force
])
def test_driver_calling_sequence_matches_the_oracle(dense, orc, driver_exe, tmp_path, bench, split,
                                                    recon, ni, nj):
    nsteps = 3
    out = tmp_path / "state.bin"
    r = subprocess.run([str(driver_exe), str(bench), str(split), str(recon), str(ni), str(nj),
                        str(nsteps), "1", str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    raw = np.fromfile(out, dtype=np.float64)
    nip, njp = ni + 8, nj + 8
    cons = raw[:nip * njp * 4].reshape((nip, njp, 4), order="F")
    t, dt = raw[-2], raw[-1]
    cfg = dense.config_default(ni=ni, nj=nj, benchmark=bench, splitting=split, recon=recon, cfl=0.5,
                               var_eps=5.0, var_xc=5.0, var_yc=5.0)
    o = orc.OracleSolver(cfg)
    o.steps(nsteps)
    ref, _ = o.get_state()
    np.testing.assert_array_equal(interior(cons), interior(ref))
    assert t == o.scalars()["time"] and dt == o.scalars()["dt"]
