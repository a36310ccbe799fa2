"""fc_dpcg_noalloc -- the Jacobi-PCG solve on the library's static scratch,
for callers that may not allocate device memory while they solve -- checked
on two calls in a row:
  - against the oracle's dpcg (the CPU restatement of the reference): the
    same iteration count, the same initial residual, the converged field
    within TOL_FIELD;
  - against the allocating entry point fc_csrsolve("dpcg"), which runs the
    same kernel on the same grid: bit for bit;
  - the library's own allocation counter does not move during either call,
    and the device's free memory does not change during the second.
The file name keeps it last in collection order, so it also runs after every
other GPU test in the same process."""
import numpy as np
import pytest

from conftest import load_fcgpu

pytestmark = pytest.mark.gpu

TOL_FIELD = 1e-8       # converged fields: max |x - x_ref| <= TOL_FIELD * max |x_ref|
TOL_RES0 = 1e-12       # initial L1 residual, relative (summation order only)


def test_noalloc_dpcg_matches_oracle_and_csrsolve():
    torch = pytest.importorskip("torch")
    import gpu_cases
    import oracle_lib
    fc = load_fcgpu()
    _, _, oc = gpu_cases.mesh_case("noalloc_hex", 14, 11, 9)
    ia, ja, a, dg, b = gpu_cases.laplacian_system(oc, 0b1)
    n, nnz = len(ia) - 1, len(ja)
    x_orc, _, info_orc, st_orc = oracle_lib.solve("dpcg", ia, ja, a, dg, np.zeros(n), b, 5000, 0.0, 1e-10)
    assert st_orc == 0
    itr_orc, res0_orc = int(info_orc[0]), float(info_orc[1])
    ctx = fc.Context(0)
    try:
        x_cs, _, info_cs, st_cs = ctx.csrsolve("dpcg", ia, ja, a, dg, np.zeros(n), b, 5000, 0.0, 1e-10)
        assert st_cs == fc.FC_OK
        dev = torch.device("cuda:0")
        t_ia = torch.from_numpy((ia - 1).astype(np.int32)).to(dev)
        t_ja = torch.from_numpy((ja - 1).astype(np.int32)).to(dev)
        t_dg = torch.from_numpy((dg - 1).astype(np.int32)).to(dev)
        t_a = torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(dev)
        t_b = torch.from_numpy(np.ascontiguousarray(b, dtype=np.float64)).to(dev)
        x = torch.zeros(n, dtype=torch.float64, device=dev)
        scale = np.abs(x_orc).max()
        for call in range(2):
            x.zero_()
            torch.cuda.synchronize()
            free0 = torch.cuda.mem_get_info(0)[0]
            allocs0 = fc.device_alloc_count()
            st, info = ctx.dpcg_noalloc(n, nnz, t_ia, t_ja, t_a, t_dg, x, t_b, 5000, 0.0, 1e-10)
            allocs1 = fc.device_alloc_count()
            free1 = torch.cuda.mem_get_info(0)[0]
            xs = x.cpu().numpy()
            assert st == fc.FC_OK, f"call {call}: status {st}"
            assert allocs1 == allocs0, f"call {call}: the library allocated or freed {allocs1 - allocs0} times"
            # against the oracle
            assert info.itr_used == itr_orc, (call, info.itr_used, itr_orc)
            assert abs(info.res0_l1 - res0_orc) <= TOL_RES0 * res0_orc
            err = np.abs(xs - x_orc).max()
            assert err <= TOL_FIELD * scale, f"call {call}: max |x - x_oracle| {err:.3e} vs {scale:.3e}"
            # against the allocating entry point: same kernel, same grid
            assert info.itr_used == info_cs.itr_used
            assert np.array_equal(xs, x_cs), f"call {call}: differs from fc_csrsolve('dpcg')"
            if call == 1:
                assert free1 == free0, f"free device memory changed by {free0 - free1} bytes"
    finally:
        ctx.close()


def test_noalloc_dpcg_rejects_bad_sizes():
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
        # ia[n] must equal nnz: a one-row system whose ia ends at 0
        ia = torch.zeros(2, dtype=torch.int32, device=dev)
        with pytest.raises(fc.FcError) as e:
            ctx.dpcg_noalloc(1, 1, ia, one_i, one_d, one_i, one_d, one_d, 10, 0.0, 1e-8)
        assert e.value.code == fc.FC_ERR_BAD_INPUT and "ia[n] == nnz" in str(e.value)
    finally:
        ctx.close()
