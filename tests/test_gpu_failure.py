"""Failure detection on the GPU without a fault: every look-back wait of the
library is bounded. A wait whose predecessor never publishes (a state word
nothing writes) runs out after the schedule's lookbackSpinLimit polls, sets
TC_DEVERR_LOOKBACK_TIMEOUT in the context's error word and returns; the host
reads the bit with tc_read_device_errors and the context stays usable: the
next frame at the default limit matches the oracle."""
import time

import pytest

from tests.conftest import cuda_available
from tests.parity import assert_same, vertex_tolerance
from vk_tessellated_clusters_gb300 import layouts as L
from vk_tessellated_clusters_gb300 import scene as S

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not cuda_available(), reason="needs a CUDA GPU")]


@pytest.fixture(scope="module")
def pipe():
    from vk_tessellated_clusters_gb300.pipeline import TessellationPipeline
    sc = S.scene_batched(num_instances=64, map_size=64)
    caps = L.default_caps(visible_bits=16, part_bits=18, split_bits=14, vertex_bits=22, megs=256)
    p = TessellationPipeline(sc, caps, L.FLAG_CULLING | L.FLAG_WRITE_FULLCLUSTERS)
    p.set_cameras(S.camera_orbit(5))
    yield p
    p.close()


def test_wait_for_a_published_predecessor_returns_its_prefix(pipe):
    pipe.set_schedule({"lookbackSpinLimit": 1})
    assert pipe.lookback_probe(published=True) == 7
    assert pipe.device_errors() == 0
    pipe.set_schedule({"lookbackSpinLimit": 0})


def test_wait_that_nothing_ends_times_out_after_one_poll(pipe):
    pipe.set_schedule({"lookbackSpinLimit": 1})
    t0 = time.perf_counter()
    assert pipe.lookback_probe(published=False) == 0
    assert time.perf_counter() - t0 < 5.0
    assert pipe.device_errors() & L.DEVERR_LOOKBACK_TIMEOUT
    assert pipe.device_errors() == 0  # reading clears the word
    pipe.set_schedule({"lookbackSpinLimit": 0})


def test_default_limit_ends_the_wait_within_seconds(pipe):
    """2^22 polls with back-off: about a second, then the error bit."""
    assert pipe.schedule()["lookbackSpinLimit"] == 0
    t0 = time.perf_counter()
    assert pipe.lookback_probe(published=False) == 0
    dt = time.perf_counter() - t0
    assert dt < 30.0, dt
    assert pipe.device_errors() & L.DEVERR_LOOKBACK_TIMEOUT


def test_frame_with_one_poll_returns_and_next_frame_matches_oracle(pipe, oracle):
    """A whole multi-tile frame with one poll per wait: every launch returns
    (no hang), the error word holds at most the timeout bit; back at the
    default limit the same context builds the frame exactly like the oracle."""
    sc = pipe.scene
    pipe.set_schedule({"lookbackSpinLimit": 1})
    for mode in ("batched", "graph"):
        pipe.build(mode)
        pipe.torch.cuda.synchronize()
        assert pipe.device_errors() & ~L.DEVERR_LOOKBACK_TIMEOUT == 0
    pipe.set_schedule({"lookbackSpinLimit": 0})
    st, _ = oracle.frame(sc, S.camera_orbit(5), pipe.caps, pipe.flags)
    want = st.outputs(oracle.entries)
    for mode in ("batched", "graph"):
        pipe.build(mode)
        got = pipe.outputs()
        assert pipe.device_errors() == 0
        assert_same(got, want, f"after timeout, {mode}", vertex_tol=vertex_tolerance(sc))
