"""fc_dpcg_noalloc -- the Jacobi-PCG solve on the library's static scratch,
allocating nothing -- against the allocating entry point fc_csrsolve("dpcg")
on the same system and start: two calls in a row, each within the
converged-field tolerance, and the second leaves the device's free memory
unchanged.  The file name keeps it last in collection order, so it also runs
after every other GPU test in the same process."""
import numpy as np
import pytest

from conftest import load_fcgpu

pytestmark = pytest.mark.gpu

TOL_FIELD = 1e-8       # converged fields: max |x - x_ref| <= TOL_FIELD * max |x_ref|
TOL_RES0 = 1e-12       # initial residual (same kernel code, possibly another grid size)
ITR_SLACK = 2          # iteration counts may differ by reduction order only


def test_noalloc_dpcg_matches_csrsolve():
    torch = pytest.importorskip("torch")
    import gpu_cases
    fc = load_fcgpu()
    _, _, oc = gpu_cases.mesh_case("noalloc_hex", 14, 11, 9)
    ia, ja, a, dg, b = gpu_cases.laplacian_system(oc, 0b1)
    n, nnz = len(ia) - 1, len(ja)
    ctx = fc.Context(0)
    try:
        x_ref, _, info_ref, st_ref = ctx.csrsolve("dpcg", ia, ja, a, dg, np.zeros(n), b, 5000, 0.0, 1e-10)
        assert st_ref == fc.FC_OK
        dev = torch.device("cuda:0")
        t_ia = torch.from_numpy((ia - 1).astype(np.int32)).to(dev)
        t_ja = torch.from_numpy((ja - 1).astype(np.int32)).to(dev)
        t_dg = torch.from_numpy((dg - 1).astype(np.int32)).to(dev)
        t_a = torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(dev)
        t_b = torch.from_numpy(np.ascontiguousarray(b, dtype=np.float64)).to(dev)
        x = torch.zeros(n, dtype=torch.float64, device=dev)
        scale = np.abs(x_ref).max()
        for call in range(2):
            x.zero_()
            torch.cuda.synchronize()
            free0 = torch.cuda.mem_get_info(0)[0]
            st, info = ctx.dpcg_noalloc(n, nnz, t_ia, t_ja, t_a, t_dg, x, t_b, 5000, 0.0, 1e-10)
            free1 = torch.cuda.mem_get_info(0)[0]
            xs = x.cpu().numpy()
            assert st == fc.FC_OK, f"call {call}: status {st}"
            assert abs(info.itr_used - info_ref.itr_used) <= ITR_SLACK, (call, info.itr_used, info_ref.itr_used)
            assert abs(info.res0_l1 - info_ref.res0_l1) <= TOL_RES0 * info_ref.res0_l1
            err = np.abs(xs - x_ref).max()
            assert err <= TOL_FIELD * scale, f"call {call}: max |dx| {err:.3e} vs {scale:.3e}"
            if call == 1:
                assert free1 == free0, f"free device memory changed by {free0 - free1} bytes"
    finally:
        ctx.close()


def test_noalloc_dpcg_rejects_oversize():
    torch = pytest.importorskip("torch")
    fc = load_fcgpu()
    ctx = fc.Context(0)
    try:
        dev = torch.device("cuda:0")
        one_i = torch.zeros(2, dtype=torch.int32, device=dev)
        one_d = torch.zeros(2, dtype=torch.float64, device=dev)
        n = fc.FC_NOALLOC_MAX_N + 1
        with pytest.raises(fc.FcError) as e:
            ctx.dpcg_noalloc(n, n, one_i, one_i, one_d, one_i, one_d, one_d, 10, 0.0, 1e-8)
        assert e.value.code == fc.FC_ERR_BAD_INPUT and "FC_NOALLOC_MAX_N" in str(e.value)
    finally:
        ctx.close()
