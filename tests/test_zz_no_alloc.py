"""pflbm_reduce_fields_noalloc: the diagnostics reduction over caller-owned
device fields, with its scratch in a file-scope device array instead of an
allocation. Checked through the C ABI against pflbm_reduce (the allocating
entry point, which reduces the simulation's own fields) on consecutive calls,
including a call over fewer z planes after one over more, so rows left in the
shared scratch by an earlier call cannot leak into a result.

Tolerance: rel 1e-10, the FP64-path parity bar of the other GPU tests (both
reduce the same float32 values in FP64, in a different summation order);
maxima and node counts exactly.
"""
import ctypes

import numpy as np
import pytest

FIELDS = ("rho", "ux", "uy", "uz", "phi")
RTOL = 1e-10


def _noalloc(pflbm, torch, host_fields, nx, ny, nz):
    lib = pflbm.load_library()
    dev = {f: torch.from_numpy(np.ascontiguousarray(host_fields[f])).to("cuda") for f in FIELDS}
    out = torch.zeros(ctypes.sizeof(pflbm.Diag), dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.pflbm_reduce_fields_noalloc(*(dev[f].data_ptr() for f in FIELDS), nx, ny, nz, stream, out.data_ptr())
    assert rc == 0, lib.pflbm_last_error().decode()
    torch.cuda.synchronize()
    return pflbm.Diag.from_buffer_copy(out.cpu().numpy().tobytes())


def _compare(got, want):
    scale_m = want.rho_mass * max(want.max_speed, 1e-30)
    assert got.step == 0
    assert got.phi_mass == pytest.approx(want.phi_mass, rel=RTOL)
    assert got.rho_mass == pytest.approx(want.rho_mass, rel=RTOL)
    for k in range(3):
        assert abs(got.momentum[k] - want.momentum[k]) <= RTOL * scale_m, k
    assert got.max_speed == want.max_speed
    assert (got.n_in, got.n_out, got.nonfinite) == (want.n_in, want.n_out, want.nonfinite)
    assert got.rho_in == pytest.approx(want.rho_in, rel=RTOL)
    assert got.rho_out == pytest.approx(want.rho_out, rel=RTOL)
    assert got.laplace_dp == pytest.approx(want.laplace_dp, rel=1e-8, abs=1e-12)


def _state(sim):
    return {f: sim.get_field(f) for f in FIELDS}


@pytest.mark.gpu
def test_noalloc_reduce_matches_pflbm_reduce(pflbm):
    torch = pytest.importorskip("torch")
    jet = pflbm.config_reference(pflbm.CASE_JET, pflbm.VS_D3Q19)  # 64 x 64 x 128: 126 interior planes
    drop = pflbm.preset("droplet64")  # 62 interior planes
    with pflbm.Simulation(jet) as s:
        s.step(20)
        want1, f1 = s.reduce(), _state(s)
        s.step(20)
        want2, f2 = s.reduce(), _state(s)
    got1 = _noalloc(pflbm, torch, f1, int(jet.nx), int(jet.ny), int(jet.nz))
    got2 = _noalloc(pflbm, torch, f2, int(jet.nx), int(jet.ny), int(jet.nz))
    _compare(got1, want1)
    _compare(got2, want2)
    assert got1.momentum[2] != got2.momentum[2]  # two different states
    with pflbm.Simulation(drop) as s:
        s.step(10)
        want3, f3 = s.reduce(), _state(s)
    got3 = _noalloc(pflbm, torch, f3, int(drop.nx), int(drop.ny), int(drop.nz))
    _compare(got3, want3)


@pytest.mark.gpu
def test_noalloc_reduce_allocates_nothing_and_refuses_host_memory(pflbm):
    """The property the entry point exists for: after a first call (which
    loads the library's kernels and the scratch array into the context),
    further calls leave the device's free memory (cudaMemGetInfo) exactly
    unchanged. A host buffer passed as a field is refused with
    PFLBM_ERR_INVALID_ARG before any kernel runs."""
    torch = pytest.importorskip("torch")
    lib = pflbm.load_library()
    cfg = pflbm.config_reference(pflbm.CASE_JET, pflbm.VS_D3Q19)
    with pflbm.Simulation(cfg) as s:
        s.step(10)
        want, host = s.reduce(), _state(s)
    nx, ny, nz = int(cfg.nx), int(cfg.ny), int(cfg.nz)
    dev = {f: torch.from_numpy(np.ascontiguousarray(host[f])).to("cuda") for f in FIELDS}
    out = torch.zeros(ctypes.sizeof(pflbm.Diag), dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    args = [dev[f].data_ptr() for f in FIELDS]

    def call(ptrs):
        return lib.pflbm_reduce_fields_noalloc(*ptrs, nx, ny, nz, stream, out.data_ptr())

    assert call(args) == 0, lib.pflbm_last_error().decode()  # warm-up
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(5):
        assert call(args) == 0, lib.pflbm_last_error().decode()
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    assert free1 == free0, (free0, free1)
    _compare(pflbm.Diag.from_buffer_copy(out.cpu().numpy().tobytes()), want)
    hbuf = np.ascontiguousarray(host["rho"])
    rc = call([hbuf.ctypes.data] + args[1:])
    assert rc == 1, rc  # PFLBM_ERR_INVALID_ARG
    assert "device memory" in lib.pflbm_last_error().decode()


def test_noalloc_reduce_rejects_too_many_planes(pflbm):
    """nz - 2 above PFLBM_NOALLOC_MAX_PLANES (4096) is refused before any CUDA call."""
    lib = pflbm.load_library()
    fake = ctypes.c_void_p(16)
    rc = lib.pflbm_reduce_fields_noalloc(fake, fake, fake, fake, fake, 8, 8, 4099, None, fake)
    assert rc == 1  # PFLBM_ERR_INVALID_ARG
    assert "PFLBM_NOALLOC_MAX_PLANES" in lib.pflbm_last_error().decode()
    assert lib.pflbm_reduce_fields_noalloc(fake, fake, fake, fake, fake, 8, 8, 4098, None, None) == 1
