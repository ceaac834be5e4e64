"""The ctypes mirror of sxsg_request matches the C struct's layout
(compiled with gcc from include/fmftsaxs_gb300.h; no GPU needed)."""
import ctypes as C
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SRC = r'''
#include <stddef.h>
#include <stdio.h>
#include "fmftsaxs_gb300.h"
#define F(x) printf("%s %zu\n", #x, offsetof(sxsg_request, x));
int main(void)
{
	printf("size %zu\n", sizeof(sxsg_request));
	F(A) F(B) F(keyA) F(keyB) F(qvals) F(qnum) F(zvals) F(znum) F(L) F(a) F(mult) F(peak) F(c1grid) F(n1)
	F(c2grid) F(n2) F(index) F(n) F(skip) F(fit_mode) F(precision)
	return 0;
}
'''


def test_request_struct_layout(tmp_path):
    import libfmftsaxs_gb300 as g
    src = tmp_path / "lay.c"
    src.write_text(SRC)
    exe = tmp_path / "lay"
    subprocess.check_call(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    out = dict(line.split() for line in subprocess.check_output([str(exe)], text=True).splitlines())
    assert int(out["size"]) == C.sizeof(g._Request)
    for name, _ in g._Request._fields_:
        assert int(out[name]) == getattr(g._Request, name).offset, name
