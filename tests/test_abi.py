"""C-ABI checks that need no GPU: the library loads, exports every function
declared in include/nqs/*.h, the ctypes struct mirrors match the C layouts,
and with no device the entry points fail cleanly instead of computing on the
CPU."""
import ctypes as C
import os
import sys
import re
import subprocess
import tempfile

import pytest

import spin_based_neural_network_gb300 as pkg
from spin_based_neural_network_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include", "nqs")


def declared_functions():
    names = set()
    for h in os.listdir(INC):
        txt = open(os.path.join(INC, h)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b(nqs_\w+)\s*\(", txt, flags=re.M):
            if "static inline" in txt[max(0, m.start() - 40):m.start() + 20]:
                continue
            names.add(m.group(1))
    return sorted(n for n in names if not n.endswith("_t"))


@pytest.fixture(scope="module")
def lib():
    pkg.build()
    return pkg.lib()


def test_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) > 50
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_struct_layouts_match_c(tmp_path):
    src = tmp_path / "layout.c"
    src.write_text("""
#include <stdio.h>
#include <stddef.h>
#include "nqs/nqs_gpu.h"
#include "nqs/nqs_marshall.h"
#include "nqs/nqs_symproj.h"
#include "nqs/nqs_translation.h"
#include "nqs/nqs_lanczos.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\\n", sizeof(nqs_config_t), offsetof(nqs_config_t, sr_cg_tol),
         offsetof(nqs_config_t, rng_seed), sizeof(nqs_sr_step_info_t), sizeof(nqs_gpu_options_t),
         sizeof(nqs_marshall_wrapper_t), sizeof(nqs_symproj_wrapper_t), sizeof(nqs_gpu_step_stats_t),
         sizeof(nqs_translation_wrapper_t), sizeof(lanczos_result_t), offsetof(lanczos_result_t, residual_norm));
  return 0;
}
""")
    exe = tmp_path / "layout"
    subprocess.check_call(["gcc", "-std=c11", "-I" + os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    got = [int(x) for x in subprocess.check_output([str(exe)]).split()]
    from spin_based_neural_network_gb300 import nqs
    want = [C.sizeof(abi.NqsConfig), abi.NqsConfig.sr_cg_tol.offset, abi.NqsConfig.rng_seed.offset,
            C.sizeof(abi.StepInfo), C.sizeof(abi.GpuOptions), C.sizeof(abi.MarshallWrapper),
            C.sizeof(abi.SymprojWrapper), C.sizeof(nqs.StepStats), C.sizeof(abi.TranslationWrapper),
            C.sizeof(abi.LanczosResult), abi.LanczosResult.residual_norm.offset]
    assert got == want


def test_config_layout_matches_upstream_header(tmp_path):
    """nqs_config_t must stay byte-identical to the upstream struct."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import link_upstream_tests as LU
    ref = LU.default_reference()
    up = os.path.join(ref, "include") if ref else ""
    if not ref or not os.path.isdir(up):
        pytest.skip("upstream headers not mounted")
    src = tmp_path / "u.c"
    src.write_text("""
#include <stdio.h>
#include <stddef.h>
#include "nqs/nqs_optimizer.h"
int main(void){printf("%zu %zu %zu\\n", sizeof(nqs_config_t), offsetof(nqs_config_t, sr_cg_tol),
 sizeof(nqs_sr_step_info_t)); return 0;}
""")
    outs = []
    for inc in (up, os.path.join(ROOT, "include")):
        exe = tmp_path / ("u%d" % len(outs))
        subprocess.check_call(["gcc", "-std=c11", "-I" + inc, str(src), "-o", str(exe)])
        outs.append(subprocess.check_output([str(exe)]))
    assert outs[0] == outs[1]


@pytest.mark.skipif(os.path.exists("/dev/nvidia0"), reason="checks the no-device behaviour")
def test_no_device_fails_loudly(lib):
    from spin_based_neural_network_gb300 import nqs
    cfg = abi.config_defaults(ansatz=abi.ANSATZ_RBM, rbm_hidden_units=4)
    h = lib.nqs_ansatz_create(C.byref(cfg), 4)
    assert not h
    assert "no CUDA device" in nqs.last_error()


def test_c_header_compiles_as_c11_and_cxx(tmp_path):
    for comp, std in (("gcc", "-std=c11"), ("g++", "-std=c++17")):
        src = tmp_path / ("h." + ("c" if comp == "gcc" else "cpp"))
        src.write_text('#include "nqs/nqs_gpu.h"\n#include "nqs/nqs_gradient.h"\n'
                       '#include "nqs/nqs_marshall.h"\n#include "nqs/nqs_symproj.h"\n'
                       '#include "nqs/nqs_optimizer.h"\n#include "nqs/nqs_translation.h"\n'
                       '#include "nqs/nqs_lanczos.h"\nint main(void){return 0;}\n')
        subprocess.check_call([comp, std, "-Wall", "-Wextra", "-Werror", "-I" + os.path.join(ROOT, "include"),
                               str(src), "-o", str(tmp_path / "h")])
