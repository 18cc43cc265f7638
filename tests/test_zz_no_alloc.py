"""The allocation-free entry point, pdpd_step_noalloc, called through the C ABI.

It serves callers that cannot allocate device memory -- a framework that owns all device
memory through its own pool, or a loop that cannot pay the synchronisation cudaMalloc and
cudaFree may cause -- so it keeps its scratch in a fixed array inside the library.  Its result must equal the
ordinary entry points' (pdpd_attach + pdpd_run, FP64 engine) bit for bit, the FP64
engine's tolerance, and stay equal on a second call that reuses the scratch array left
behind by the first.  This file is named to be collected last.
"""

import numpy as np
import pytest

import pdpd_engine as E
import pdpd_world as W

pytestmark = pytest.mark.gpu


def _device_arrays(world):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    x = torch.tensor(world.x, dtype=torch.float64, device=dev).contiguous()
    v = torch.tensor(world.v, dtype=torch.float64, device=dev).contiguous()
    f = torch.tensor(world.f, dtype=torch.float64, device=dev).contiguous()
    h = torch.tensor(world.hashes().astype(np.int64), dtype=torch.int64).to(torch.int32).to(dev)
    return x, v, f, h


@pytest.mark.parametrize("side,density", [(10, 3), (32, 2)], ids=["3000_beads", "at_the_limit"])
def test_step_noalloc_matches_run_on_two_calls(side, density):
    """Two calls in a row equal pdpd_run bit for bit; 32^3 at density 2 fills the scratch
    exactly (65,536 beads, 32,768 cells)."""
    torch = pytest.importorskip("torch")
    world = W.make_water(side, seed=6, dt=0.02, density=density)
    if side == 32:
        assert world.n_beads == E.NOALLOC_MAX_BEADS and 32 ** 3 == E.NOALLOC_MAX_CELLS
    x, v, f, h = _device_arrays(world)

    ref = world.copy()
    eng = E.GB300DPDEngine("fp64", device=0)
    eng.Attach(ref)

    t = world.t
    for call in range(2):
        steps = 4
        E.step_noalloc(world, x.data_ptr(), v.data_ptr(), f.data_ptr(), h.data_ptr(), steps, t=t)
        t += steps
        eng.Run(steps)
        assert ref.t == t
        assert np.array_equal(x.cpu().numpy(), ref.x), f"x differs after call {call + 1}"
        assert np.array_equal(v.cpu().numpy(), ref.v), f"v differs after call {call + 1}"
        assert np.array_equal(f.cpu().numpy(), ref.f), f"f differs after call {call + 1}"


def test_step_noalloc_reports_a_bead_lost_in_the_first_step():
    """A bead that leaves the box in step 1 of a 4-step call (it starts 2.5 box sides out, so
    one periodic wrap does not bring it back) is reported at the end of the call, although
    steps 2-4 run normally."""
    world = W.make_water(8, seed=3, dt=0.02)
    world.x[17, 0] = 2.5 * world.box[0]
    x, v, f, h = _device_arrays(world)
    with pytest.raises(RuntimeError, match="PDPD_E_BEAD_LOST"):
        E.step_noalloc(world, x.data_ptr(), v.data_ptr(), f.data_ptr(), h.data_ptr(), 4)
    # The next call starts with a clear error word.
    good = W.make_water(8, seed=3, dt=0.02)
    x, v, f, h = _device_arrays(good)
    E.step_noalloc(good, x.data_ptr(), v.data_ptr(), f.data_ptr(), h.data_ptr(), 2)


def test_step_noalloc_rejects_oversized_and_bonded_worlds():
    big = W.make_water(40, seed=1)  # 192,000 beads > the fixed scratch size
    with pytest.raises(RuntimeError, match="PDPD_E_NOMEM"):
        E.step_noalloc(big, 1, 1, 1, 1, 1)
    bonded = W.make_polymer_box(6, chain_fraction=0.1)
    with pytest.raises(RuntimeError, match="bonds"):
        E.step_noalloc(bonded, 1, 1, 1, 1, 1)
