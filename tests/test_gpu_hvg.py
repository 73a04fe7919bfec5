"""GPU HVG statistics (brisc_gb300.hvg, brisc/hvg.pyx) against the reference's
own outputs (tests/golden/hvg.npz) and the oracle, bit for bit."""
import numpy as np
import pytest
import scipy.sparse as sp

from brisc_gb300 import hvg
from oracle import hvg as oh
from test_oracle import HVG_TAGS, hvg_case

pytestmark = pytest.mark.gpu


def _run(form, d, ix, ip, cells, mask, nc, g, clip, device):
    """The four entry points on host arrays, or on CUDA tensors."""
    import torch

    def put(a):
        return torch.from_numpy(np.ascontiguousarray(a)).cuda() if device else a

    def out(n, dt):
        a = np.zeros(n, dt)
        return put(a)

    def back(a):
        return a.cpu().numpy() if device else a

    # nonzero counts: uint32 on the host; an int32 CUDA tensor holds the same
    # 32-bit words on the device
    m, v = out(g, np.float32), out(g, np.float32)
    c = out(g, np.int32 if device else np.uint32)
    b, q = out(g, np.float32), out(g, np.float32)
    D, IX, IP, CL = put(d), put(ix), put(ip), put(clip)
    if form == "csr":
        hvg.gene_mean_and_variance_csr(D, IX, IP, put(cells), nc, g, m, v, c, 8)
        hvg.clipped_sum_csr(D, IX, IP, nc, g, put(cells), CL, b, q, 8)
    else:
        hvg.gene_mean_and_variance_csc(D, IX, IP, put(mask), nc, g, m, v, c, 8)
        hvg.clipped_sum_csc(D, IX, IP, put(mask), CL, b, q, 8)
    if device:
        torch.cuda.synchronize()
    cc = back(c)
    return back(m), back(v), cc.view(np.uint32), back(b), back(q)


@pytest.mark.parametrize("device", [False, True])
@pytest.mark.parametrize("sub", ["all", "sub"])
@pytest.mark.parametrize("form", ["csr", "csc"])
@pytest.mark.parametrize("tag", HVG_TAGS)
def test_hvg_matches_reference(cuda, golden, tag, form, sub, device):
    z = golden("hvg")
    n, g = int(z["n"]), int(z["g"])
    d, ix, ip = hvg_case(z, form, tag)
    if device and d.dtype == np.uint32:
        pytest.skip("torch keeps no uint32 CUDA tensors on every version")
    cells = z["cells"] if sub == "sub" else np.zeros(0, np.int64)
    mask = z["mask"] if sub == "sub" else np.zeros(0, np.int8)
    nc = len(cells) if sub == "sub" else n
    got = _run(form, d, ix, ip, cells, mask, nc, g, z["clip"], device)
    key = f"{form}_{tag}_{sub}"
    for a, name in zip(got, ("mean", "var", "nnz", "bsum", "bsq")):
        assert np.array_equal(a, z[f"{key}_{name}"]), name


def _random(n, g, dtype, itype, seed):
    rng = np.random.default_rng(seed)
    X = (rng.random((n, g)) < 0.08) * rng.integers(1, 300, (n, g))
    X[rng.random((n, g)) < 0.001] = 40000  # above every clip value
    A = sp.csr_matrix(X)
    B = sp.csc_matrix(X)
    A.sort_indices()
    B.sort_indices()
    return ((A.data.astype(dtype), A.indices.astype(itype), A.indptr.astype(itype)),
            (B.data.astype(dtype), B.indices.astype(itype), B.indptr.astype(itype)))


@pytest.mark.parametrize("itype", [np.int32, np.int64])
@pytest.mark.parametrize("dtype", [np.uint16, np.int32, np.uint32, np.int64,
                                   np.uint64, np.float32, np.float64])
def test_hvg_every_value_type(cuda, dtype, itype):
    n, g = 1500, 300
    csr, csc = _random(n, g, dtype, itype, 7)
    rng = np.random.default_rng(8)
    cells = np.sort(rng.choice(n, 500, replace=False)).astype(np.int64)
    mask = np.zeros(n, np.int8)
    mask[cells] = 1
    clip = (rng.random(g) * 200 + 1).astype(np.float32)
    for sub in (False, True):
        c = cells if sub else np.zeros(0, np.int64)
        mk = mask if sub else np.zeros(0, np.int8)
        nc = len(cells) if sub else n
        for form, (d, ix, ip) in (("csr", csr), ("csc", csc)):
            got = _run(form, d, ix, ip, c, mk, nc, g, clip, False)
            if form == "csr":
                want = (*oh.gene_mean_and_variance_csr(d, ix, ip, c, nc, g),
                        *oh.clipped_sum_csr(d, ix, ip, nc, g, c, clip))
            else:
                want = (*oh.gene_mean_and_variance_csc(d, ix, ip, mk, nc, g),
                        *oh.clipped_sum_csc(d, ix, ip, mk, clip))
            for a, w, name in zip(got, want, ("mean", "var", "nnz", "bsum", "bsq")):
                assert np.array_equal(a, w), (form, sub, name)


def test_hvg_many_genes_global_accumulators(cuda):
    """More genes than one CTA's shared accumulators hold (4096): the CSR
    kernels add straight into global memory."""
    n, g = 800, 6000
    csr, csc = _random(n, g, np.uint32, np.int32, 9)
    d, ix, ip = csr
    clip = np.full(g, 150.5, np.float32)
    got = _run("csr", d, ix, ip, np.zeros(0, np.int64), np.zeros(0, np.int8), n, g,
               clip, False)
    want = (*oh.gene_mean_and_variance_csr(d, ix, ip, np.zeros(0, np.int64), n, g),
            *oh.clipped_sum_csr(d, ix, ip, n, g, np.zeros(0, np.int64), clip))
    for a, w in zip(got, want):
        assert np.array_equal(a, w)


def test_hvg_out_of_range_index_rejected(cuda):
    """A gene index past num_dataset_genes is skipped by the kernel and
    reported as a ValueError (the reference would write out of bounds)."""
    ip = np.array([0, 2, 3], np.int32)
    ix = np.array([0, 5, 1], np.int32)  # gene 5 of 3
    d = np.array([1, 2, 3], np.uint32)
    m, v, c = np.zeros(3, np.float32), np.zeros(3, np.float32), np.zeros(3, np.uint32)
    with pytest.raises(ValueError, match="out of bounds"):
        hvg.gene_mean_and_variance_csr(d, ix, ip, np.zeros(0, np.int64), 2, 3, m, v, c, 1)
    mask = np.ones(1, np.int8)  # cell 1 is past the mask
    with pytest.raises(ValueError, match="out of bounds"):
        hvg.gene_mean_and_variance_csc(d, np.array([0, 1, 0], np.int32), ip, mask, 2, 2,
                                       m, v, c, 1)


def test_hvg_called_as_single_cell_calls_it(cuda, golden):
    """The keyword calls of SingleCell's HVG step (brisc/single_cell.py:
    11320-11395): CSR with an int64 cell list and num_cells = its length,
    CSC with a boolean cell mask."""
    z = golden("hvg")
    n, g = int(z["n"]), int(z["g"])
    cells = z["cells"]
    for form in ("csr", "csc"):
        d, ix, ip = hvg_case(z, form, "float32_int32")
        mean, var = np.zeros(g, np.float32), np.zeros(g, np.float32)
        nz = np.zeros(g, np.uint32)
        b, q = np.empty(g, np.float32), np.empty(g, np.float32)
        if form == "csr":
            hvg.gene_mean_and_variance_csr(
                data=d, indices=ix, indptr=ip, cell_indices=cells,
                num_cells=len(cells), num_dataset_genes=g, mean=mean, var=var,
                nonzero_count=nz, num_threads=4)
            hvg.clipped_sum_csr(
                data=d, indices=ix, indptr=ip, num_cells=len(cells),
                num_dataset_genes=g, cell_indices=cells, clip_val=z["clip"],
                batch_counts_sum=b, squared_batch_counts_sum=q, num_threads=4)
        else:
            mask = z["mask"].astype(bool)
            hvg.gene_mean_and_variance_csc(
                data=d, indices=ix, indptr=ip, cell_mask=mask,
                num_cells=int(mask.sum()), num_dataset_genes=g, mean=mean, var=var,
                nonzero_count=nz, num_threads=4)
            hvg.clipped_sum_csc(
                data=d, indices=ix, indptr=ip, cell_mask=mask, clip_val=z["clip"],
                batch_counts_sum=b, squared_batch_counts_sum=q, num_threads=4)
        key = f"{form}_float32_int32_sub"
        for a, name in ((mean, "mean"), (var, "var"), (nz, "nnz"), (b, "bsum"),
                        (q, "bsq")):
            assert np.array_equal(a, z[f"{key}_{name}"]), (form, name)
