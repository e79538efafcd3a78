"""GPU: behf_field_norm_noalloc, the field health check for callers that cannot allocate device memory.

Those callers (an application whose own pool already holds the GPU, or a monitoring thread that must
not stall the device with cudaFree) hand in a field and two output words they own; the entry point
uses only its fixed scratch array inside the library.  Its results must equal the context-based
behf_health on the same data, call after call, because every call reuses that scratch.
This file is collected last so that a failing run stops after every other test has run.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _health_norm(values: np.ndarray, precision: str, field: str = "szz"):
    """Sum of squares and health flag of `values` through the existing context entry point."""
    import behf
    nz, ny, nx = values.shape
    s = behf.Solver(nx, ny, nz, 5.0, 4e-4, radius=2, precision=precision, cpml_width=0,
                    scales=(1.0, 1.0, 1.0, 1.0))
    s.set_field(field, values)
    ok, norms = s.health()
    s.close()
    return ok, float(norms[behf.FIELD[field]])


def _noalloc_norm(values: np.ndarray, precision: str, pitch_pad: int, out, flag):
    import torch

    import behf
    nz, ny, nx = values.shape
    dt = {"f64": torch.float64, "f32": torch.float32, "f16": torch.float16, "bf16": torch.bfloat16}[precision]
    pitch = nx + pitch_pad
    buf = torch.full((nz, ny, pitch), float("nan"), dtype=dt, device="cuda")  # padding must not be read
    buf[:, :, :nx] = torch.from_numpy(values).to(dt)
    stream = torch.cuda.current_stream()
    behf.field_norm_noalloc(buf.data_ptr(), precision, nx, ny, nz, pitch, pitch * ny, out.data_ptr(),
                            flag.data_ptr(), stream.cuda_stream)
    stream.synchronize()
    return int(flag.item()) == 0, float(out.item())


@pytest.mark.parametrize("precision", ["f64", "f32", "f16", "bf16"])
def test_noalloc_matches_health_on_two_calls(behf_lib, precision):
    import torch
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    flag = torch.full((1,), 7, dtype=torch.int32, device="cuda")
    rng = np.random.default_rng(11)
    # second call on a smaller field: the first call's leftover partial sums must not leak into it
    for shape, pad in (((40, 36, 33), 7), ((9, 23, 29), 0)):
        v = (rng.standard_normal(shape) * 3).astype(np.float32)
        ok_ref, ref = _health_norm(v, precision)
        ok, got = _noalloc_norm(v, precision, pad, out, flag)
        assert ok and ok_ref
        assert got == pytest.approx(ref, rel=1e-12)


def test_noalloc_flags_nonfinite_then_recovers(behf_lib):
    import torch
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    flag = torch.zeros(1, dtype=torch.int32, device="cuda")
    v = np.ones((12, 14, 16), np.float32)
    v[5, 6, 7] = np.inf
    ok_ref, _ = _health_norm(v, "f32")
    ok, _ = _noalloc_norm(v, "f32", 0, out, flag)
    assert not ok and not ok_ref
    v[5, 6, 7] = 2.0  # the next call starts clean although the scratch still holds the bad partial
    ok_ref, ref = _health_norm(v, "f32")
    ok, got = _noalloc_norm(v, "f32", 3, out, flag)
    assert ok and ok_ref and got == pytest.approx(ref, rel=1e-12)


@pytest.mark.parametrize("precision,top", [("f16", 65504.0), ("bf16", 3.3895313892515355e38)])
def test_noalloc_flags_saturation_like_health(behf_lib, precision, top):
    """A value at the largest finite value of the storage format is flagged by both entry points, and both
    leave it out of the norm while keeping the other cells."""
    import torch
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    flag = torch.zeros(1, dtype=torch.int32, device="cuda")
    rng = np.random.default_rng(5)
    v = rng.standard_normal((10, 12, 14)).astype(np.float32)
    v[3, 4, 5] = top
    ok_ref, ref = _health_norm(v, precision)
    ok, got = _noalloc_norm(v, precision, 2, out, flag)
    assert not ok_ref and not ok
    assert got == pytest.approx(ref, rel=1e-12) and 0 < got < 1e6


def test_noalloc_rejects_fields_beyond_its_scratch(behf_lib):
    import torch

    import behf
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    flag = torch.zeros(1, dtype=torch.int32, device="cuda")
    with pytest.raises(behf.BehfError) as e:  # 1025^3 cells > 2^30: refused before any launch
        behf.field_norm_noalloc(out.data_ptr(), "f16", 1025, 1025, 1025, 1025, 1025 * 1025, out.data_ptr(),
                                flag.data_ptr(), 0)
    assert e.value.code == -1 and "exceed" in str(e.value)
