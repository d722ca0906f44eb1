"""Host-side argument checks of the Python layer: rejected before any device
work, with the exception types the drop-in contract promises (ValueError for
bad arguments, NotImplementedError for reference features the GPU engine
routes back to the reference)."""
import numpy as np
import pytest

from oqupy_gb300 import GpuPtTempoBackend, GpuTempoBackend, PtBatch, TempoBatch


def _tempo_inst():
    D = 4
    return dict(hs_dim=2, dkmax=3, epsrel=1e-6, influences=np.ones((4, D, D), complex),
                prop1=np.eye(D), prop2=np.eye(D), rho0=np.diag([1.0, 0.0]))


def test_tempo_batch_rejects_bad_precision_and_empty_batch():
    with pytest.raises(ValueError):
        TempoBatch([_tempo_inst()], precision="fp16")
    with pytest.raises(ValueError):
        TempoBatch([], precision="mixed")


def test_pt_batch_rejects_bad_arguments():
    inst = dict(hs_dim=2, num_steps=5, dkmax=3, epsrel=1e-6, influences=np.ones((4, 4, 4), complex))
    with pytest.raises(ValueError):
        PtBatch([inst], precision="tf32")
    with pytest.raises(ValueError):
        PtBatch([])
    with pytest.raises(ValueError):
        PtBatch([dict(inst, num_steps=1)])          # min(num_steps, dkmax + 1) < 2


def test_gpu_backends_route_unsupported_reference_features():
    infl = lambda dk: np.ones((4, 4), complex)       # noqa: E731
    props = lambda step: (np.eye(4), np.eye(4))      # noqa: E731
    with pytest.raises(NotImplementedError):
        GpuTempoBackend(np.ones(4), infl, np.eye(2), props, np.ones(4), np.ones(4), 3, 1e-6,
                        config={"backend": "gb300"}, degeneracy_maps=([0], [0]))
    with pytest.raises(NotImplementedError):
        GpuTempoBackend(np.ones(4), infl, np.eye(2), props, 2 * np.ones(4), np.ones(4), 3, 1e-6,
                        config={"backend": "gb300"})
    with pytest.raises(NotImplementedError):
        GpuPtTempoBackend(2, infl, None, np.ones(4), np.ones(4), 5, 3, 1e-6, {"backend": "gb300"},
                          degeneracy_maps=([0], [0]))
    with pytest.raises(NotImplementedError):
        GpuPtTempoBackend(2, infl, None, np.ones(4), np.zeros(4), 5, 3, 1e-6, {"backend": "gb300"})


def test_bucket_tuner_alternates_then_keeps_the_faster_shape():
    from oqupy_gb300.autotune import BucketTuner
    t = BucketTuner(candidates=[(256, 56), (512, 200)], bucket_width=8)
    t.begin_chunk(5)
    assert t.tuning()
    shapes = [t.shape_for(k) for k in range(6)]
    # two trial launches per candidate, then the first candidate
    assert shapes == [(256, 56), (512, 200), (256, 56), (512, 200), (256, 56), (256, 56)]
    t.end_chunk([10.0, 14.0, 11.0, 15.0, 30.0, 30.0])   # narrow CTAs faster in the trials
    assert not t.tuning() and t.shape_for(0) == (256, 56)
    t.begin_chunk(30)                               # a new bucket is tuned again
    assert t.tuning()
    t.end_chunk([20.0, 12.0, 21.0, 13.0])
    assert t.shape_for(3) == (512, 200)
    t.begin_chunk(6)
    assert t.shape_for(1) == (256, 56)
    assert t.table() == {"bond 0-7": [256, 56], "bond 24-31": [512, 200]}
