"""The allocation-free SIR step (vg_sir_step_noalloc) against the "sir"
transition of apply!, through the C ABI.

Some callers cannot let a library allocate device memory -- a host runtime
that owns all device memory and passes pre-allocated arrays in, or code
running while another framework captures a CUDA graph.  For them the
library offers one SIR step on caller-owned buffers whose only scratch is a
fixed file-scope device table.  This test runs two such steps in a row
(ping-pong buffers) next to two apply! steps on the same graph and state,
and requires bit-identical results (tolerance 0, as every SIR test); then
two more with the largest in-degree understated (the rows beyond the table),
and checks that an in-place call and a table beyond its fixed size are
refused.
It is collected last and runs alone or after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_sir_step_noalloc_matches_apply(vh):
    import torch
    from vahana_gb300 import models
    from vahana_gb300._lib import check, lib
    n, beta, rec, seed = 3000, 0.05, 7, 21
    run = models.build_sir(n=n, degree=10, beta=beta, recovery=rec, seed=seed, n_infected=60)
    vh.finish_init(run.sim)
    rp, frm, _ = vh.read_edges(run.sim, "Contact", "Person")
    cols, _ = vh.read_agents(run.sim, "Person")
    deg = np.diff(rp)
    dev = torch.device("cuda:0")
    row_ptr = torch.tensor(rp.astype(np.uint32).view(np.int32), device=dev)
    src = torch.tensor(((frm & np.uint64((1 << 36) - 1)) - 1).astype(np.uint32).view(np.int32),
                       device=dev)
    st = [torch.tensor(cols["state"].view(np.int8), device=dev), torch.empty(n, dtype=torch.int8,
                                                                             device=dev)]
    dy = [torch.tensor(cols["days"], device=dev), torch.empty(n, dtype=torch.int32, device=dev)]
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        step = vh.num_transitions(run.sim)  # the transition number apply! uses next
        a, b = call % 2, (call + 1) % 2
        check(lib().vg_sir_step_noalloc(
            C.c_void_p(row_ptr.data_ptr()), C.c_void_p(src.data_ptr()),
            C.c_void_p(st[a].data_ptr()), C.c_void_p(dy[a].data_ptr()),
            C.c_void_p(st[b].data_ptr()), C.c_void_p(dy[b].data_ptr()),
            C.c_uint64(n), C.c_uint32(int(deg.max())), C.c_double(beta), C.c_int32(rec),
            C.c_uint64(seed), C.c_uint32(step), C.c_void_p(stream)))
        run.step()
        torch.cuda.synchronize()
        ref, _ = vh.read_agents(run.sim, "Person")
        got_s = st[b].cpu().numpy().view(np.uint8)
        got_d = dy[b].cpu().numpy()
        np.testing.assert_array_equal(got_s, ref["state"])
        np.testing.assert_array_equal(got_d, ref["days"])
    assert (got_s == 1).sum() > 0
    # a caller that understates the largest in-degree (1, then 0): rows with
    # more infected neighbours than the table covers form the same product
    # on the device; still bit-identical to apply!
    for call, kmax in ((2, 1), (3, 0)):
        step = vh.num_transitions(run.sim)
        a, b = call % 2, (call + 1) % 2
        check(lib().vg_sir_step_noalloc(
            C.c_void_p(row_ptr.data_ptr()), C.c_void_p(src.data_ptr()),
            C.c_void_p(st[a].data_ptr()), C.c_void_p(dy[a].data_ptr()),
            C.c_void_p(st[b].data_ptr()), C.c_void_p(dy[b].data_ptr()),
            C.c_uint64(n), C.c_uint32(kmax), C.c_double(beta), C.c_int32(rec),
            C.c_uint64(seed), C.c_uint32(step), C.c_void_p(stream)))
        run.step()
        torch.cuda.synchronize()
        ref, _ = vh.read_agents(run.sim, "Person")
        np.testing.assert_array_equal(st[b].cpu().numpy().view(np.uint8), ref["state"])
        np.testing.assert_array_equal(dy[b].cpu().numpy(), ref["days"])
    # an in-place step (output = input) is refused, not run half-updated
    rc = lib().vg_sir_step_noalloc(
        C.c_void_p(row_ptr.data_ptr()), C.c_void_p(src.data_ptr()),
        C.c_void_p(st[0].data_ptr()), C.c_void_p(dy[0].data_ptr()),
        C.c_void_p(st[0].data_ptr()), C.c_void_p(dy[1].data_ptr()),
        C.c_uint64(n), C.c_uint32(int(deg.max())), C.c_double(beta), C.c_int32(rec),
        C.c_uint64(seed), C.c_uint32(1), C.c_void_p(stream))
    assert rc != 0 and b"overlap" in lib().vg_last_error()
    # sizes beyond the fixed table are rejected with a clear error
    rc = lib().vg_sir_step_noalloc(
        C.c_void_p(row_ptr.data_ptr()), C.c_void_p(src.data_ptr()),
        C.c_void_p(st[0].data_ptr()), C.c_void_p(dy[0].data_ptr()),
        C.c_void_p(st[1].data_ptr()), C.c_void_p(dy[1].data_ptr()),
        C.c_uint64(n), C.c_uint32(1 << 20), C.c_double(beta), C.c_int32(rec),
        C.c_uint64(seed), C.c_uint32(1), C.c_void_p(stream))
    assert rc != 0 and b"max_in_degree" in lib().vg_last_error()
    run.close()
