"""Which tcgen05 MMA kinds the toolkit assembles for GB300 (sm_103a).

The batched engine splits its words into 8-bit digits; on sm_103a it runs
them on `tcgen05.mma kind::f16` because `kind::i8` (the INT8 tensor-core
form with TMEM accumulators) does not exist there: ptxas rejects it. This
test keeps that fact checked against the installed toolkit (no GPU needed:
nvcc only assembles).
"""
import os
import shutil
import subprocess

import pytest

SRC = r'''
#include <cstdint>
__global__ void issue(uint32_t d, uint64_t a, uint64_t b, uint32_t id) {
  asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %3, 0;\n\t"
               "tcgen05.mma.cta_group::1.kind::KIND [%0], %1, %2, %3, p;\n\t}"
               :: "r"(d), "l"(a), "l"(b), "r"(id));
}
'''


def _assemble(tmp_path, kind, arch):
    src = tmp_path / ("mma_%s_%s.cu" % (kind, arch))
    src.write_text(SRC.replace("KIND", kind))
    r = subprocess.run(
        ["nvcc", "-gencode", "arch=compute_%s,code=sm_%s" % (arch, arch),
         "-c", str(src), "-o", os.devnull], capture_output=True, text=True)
    return r.returncode, r.stdout + r.stderr


@pytest.mark.skipif(shutil.which("nvcc") is None, reason="needs nvcc")
def test_kind_i8_is_rejected_and_kind_f16_accepted_on_sm103a(tmp_path):
    rc, out = _assemble(tmp_path, "i8", "103a")
    assert rc != 0
    assert "kind::i8" in out and "not supported" in out
    rc, out = _assemble(tmp_path, "f16", "103a")
    assert rc == 0, out
