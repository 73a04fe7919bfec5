"""Served PCA requests on the GPU: each result is the same alone and in the
mix (bit-identical PCs), with several requests overlapping on the device."""
import numpy as np
import pytest

from brisc_gb300.serve import PCARequest, PCAServer, gpu_solve
from synth import nb_counts

pytestmark = pytest.mark.gpu


def _request(n, g, density, k, seed):
    c = nb_counts(n, g, seed=seed, density=density, workers=1)
    return PCARequest(c.indptr.astype(np.int32), c.indices, c.data, g, c.isf,
                      num_PCs=k, seed=seed, tag=seed)


def test_results_identical_alone_and_in_the_mix(cuda):
    import torch
    specs = [(6000, 300, 0.08, 10), (20000, 500, 0.05, 20), (3000, 200, 0.06, 8),
             (12000, 400, 0.03, 15), (9000, 250, 0.07, 12), (2500, 150, 0.05, 6)]
    reqs = [_request(n, g, d, k, seed) for seed, (n, g, d, k) in enumerate(specs)]
    alone = []
    s = torch.cuda.Stream()
    for r in reqs:
        alone.append(gpu_solve(r, s))
    with PCAServer(slots=3) as srv:
        futs = [srv.submit(r) for r in reqs]
        mixed = [f.result(timeout=300) for f in futs]
    assert srv.max_running >= 2  # requests really overlapped
    for a, m in zip(alone, mixed):
        assert m.error is None
        assert np.array_equal(a.PCs, m.result.PCs)
        assert np.array_equal(a.singular_values, m.result.singular_values)
