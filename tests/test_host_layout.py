"""Host-side ABI layout: the Python mirror of struct Wparams matches the C
layout (float4 is 16-byte aligned), checked by compiling a probe with gcc."""
import os
import subprocess
import tempfile

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_wparams_layout_matches_c():
    import ctypes

    import wltube

    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "wl_legacy.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu\n", offsetof(struct Wparams, xcm),
         offsetof(struct Wparams, Wsscal_h), offsetof(struct Wparams, worldlines),
         offsetof(struct Wparams, ng), offsetof(struct Wparams, rho2sp), sizeof(struct Wparams));
  return 0;
}
'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "p.c")
        open(c, "w").write(src)
        exe = os.path.join(d, "p")
        subprocess.check_call(["gcc", "-I" + os.path.join(ROOT, "include"),
                               "-I/usr/local/cuda/include", c, "-o", exe])
        got = [int(v) for v in subprocess.check_output([exe]).split()]
    W = wltube.Wparams
    assert got == [W.xcm.offset, W.Wsscal_h.offset, W.worldlines.offset, W.ng.offset,
                   W.rho2sp.offset, ctypes.sizeof(W)]


def test_server_structs_match_c():
    import ctypes

    import wltube

    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "wlgpu.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\n",
         offsetof(wl_request, field), offsetof(wl_request, cx), offsetof(wl_request, rho),
         offsetof(wl_request, F), offsetof(wl_request, group), offsetof(wl_request, out_err),
         sizeof(wl_request), offsetof(wl_server_config, max_requests), sizeof(wl_server_config),
         offsetof(wl_server_stats, hbm_bytes_in_use), sizeof(wl_server_stats));
  return 0;
}
'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "p.c")
        open(c, "w").write(src)
        exe = os.path.join(d, "p")
        subprocess.check_call(["gcc", "-I" + os.path.join(ROOT, "include"),
                               "-I/usr/local/cuda/include", c, "-o", exe])
        got = [int(v) for v in subprocess.check_output([exe]).split()]
    Q, G, S = wltube.Request, wltube.ServerConfig, wltube.ServerStats
    assert got == [Q.field.offset, Q.cx.offset, Q.rho.offset, Q.F.offset, Q.group.offset,
                   Q.out_err.offset, ctypes.sizeof(Q), G.max_requests.offset, ctypes.sizeof(G),
                   S.hbm_bytes_in_use.offset, ctypes.sizeof(S)]
