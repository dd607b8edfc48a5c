"""psim_final_temps_noalloc: the allocation-free final-temperature call, through the C ABI.

Its results must equal psim_final_temps on the same tallies (tolerance: exact, 0 ulp - both
run the same FP64 kernels compiled without contraction), on consecutive calls that reuse the
one fixed device scratch.  Device buffers belong to the caller; torch provides them here."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, model_path

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env(gpu):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("torch sees no CUDA device")
    torch.cuda.set_device(0)
    from psim_gb300 import api
    return api, torch


def _case(api, name):
    gold = np.load(os.path.join(GOLDEN, f"invert_{name}.npz"))
    m = api.Model(model_path(name))
    d = m.interp_desc(float(gold["eff"]))
    counts = np.ascontiguousarray(gold["counts"], dtype=np.int64)
    assert counts.shape == (d.n_sensors, d.recorded_steps)
    return m, d, counts


@pytest.mark.parametrize("name", ["bar_full", "bar_ss", "kinked_small"])
def test_two_calls_match_existing_entry_point(env, name):
    api, torch = env
    m, d, counts = _case(api, name)
    S = d.n_sensors
    second = counts[:, ::-1].copy()  # different tallies for the second call
    want1 = api.final_temps(d, counts, 1)
    want2 = api.final_temps(d, second, 0)

    e1 = torch.from_numpy(counts).cuda()
    e2 = torch.from_numpy(second).cuda()
    out1 = torch.full((S,), float("nan"), dtype=torch.float64, device="cuda")
    out2 = torch.full((S,), float("nan"), dtype=torch.float64, device="cuda")
    stream = torch.cuda.Stream()
    torch.cuda.synchronize()
    # two calls in a row on one stream, no wait between them: the second reuses the scratch
    api.final_temps_noalloc(d, e1.data_ptr(), 1, out1.data_ptr(), stream.cuda_stream)
    api.final_temps_noalloc(d, e2.data_ptr(), 0, out2.data_ptr(), stream.cuda_stream)
    stream.synchronize()
    assert np.array_equal(out1.cpu().numpy(), want1)
    assert np.array_equal(out2.cpu().numpy(), want2)
    # and once more on the legacy default stream, after the others
    out1.fill_(float("nan"))
    torch.cuda.synchronize()
    api.final_temps_noalloc(d, e1.data_ptr(), 1, out1.data_ptr(), None)
    torch.cuda.synchronize()
    assert np.array_equal(out1.cpu().numpy(), want1)
    m.close()


def test_rejects_inputs_beyond_the_scratch(env):
    api, torch = env
    m, d, counts = _case(api, "bar_ss")
    cap = api.final_temps_noalloc_max_bytes()
    assert cap == 8 << 20
    S = d.n_sensors
    K = cap // (8 * S) + 1  # S x K temperatures alone exceed the scratch
    big = torch.zeros((S, K), dtype=torch.int64, device="cuda")  # a real buffer of that shape
    out = torch.zeros((S,), dtype=torch.float64, device="cuda")
    d.recorded_steps = K
    with pytest.raises(api.PsimError) as exc:
        api.final_temps_noalloc(d, big.data_ptr(), 0, out.data_ptr(), None)
    assert exc.value.code == 4 and "scratch" in str(exc.value)
    # a rejected call enqueues nothing: a valid call pending on a stream keeps its scratch and result,
    # and the rejected call's output buffer keeps its contents
    m_ok, d_ok, counts = _case(api, "bar_ss")
    want = api.final_temps(d_ok, counts, 1)
    e_ok = torch.from_numpy(counts).cuda()
    out_ok = torch.full((S,), float("nan"), dtype=torch.float64, device="cuda")
    sentinel = torch.full((S,), -12345.0, dtype=torch.float64, device="cuda")
    stream = torch.cuda.Stream()
    torch.cuda.synchronize()
    api.final_temps_noalloc(d_ok, e_ok.data_ptr(), 1, out_ok.data_ptr(), stream.cuda_stream)
    with pytest.raises(api.PsimError) as exc:
        api.final_temps_noalloc(d, big.data_ptr(), 0, sentinel.data_ptr(), stream.cuda_stream)
    assert exc.value.code == 4
    stream.synchronize()
    assert np.array_equal(out_ok.cpu().numpy(), want)
    assert bool((sentinel == -12345.0).all())
    m_ok.close()
    # past the start step is an argument error, not a size error
    with pytest.raises(api.PsimError) as exc:
        api.final_temps_noalloc(d, big.data_ptr(), K + 1, out.data_ptr(), None)
    assert exc.value.code == 1
    torch.cuda.synchronize()
    m.close()
