"""Copy merging of the host pipeline (batch._contiguous_runs): runs of
consecutive tensors adjacent in one storage, on CPU tensors."""

import pytest


def test_contiguous_runs_of_views():
    torch = pytest.importorskip("torch")
    from fastlisaresponse_gb300.batch import _contiguous_runs

    base = torch.arange(100, dtype=torch.float64)
    views = [base[0:10], base[10:25], base[25:26], base[30:40], base[40:41]]
    runs = _contiguous_runs(views)
    assert [(a, b) for a, b, _ in runs] == [(0, 3), (3, 5)]
    assert torch.equal(runs[0][2], base[0:26]) and torch.equal(runs[1][2], base[30:41])
    # 2-D (3, n) views of one flat buffer, as host channel outputs
    flat = torch.zeros(3 * 12, dtype=torch.float64)
    outs = [flat[0:9].view(3, 3), flat[9:36].view(3, 9)]
    (a, b, span), = _contiguous_runs(outs)
    assert (a, b) == (0, 2) and span.data_ptr() == flat.data_ptr() and span.numel() == 36
    # separate storages and dtype changes break runs
    other = torch.arange(10, dtype=torch.float64)
    assert len(_contiguous_runs([base[0:10], other])) == 2
    assert len(_contiguous_runs([base[0:4], base[4:8].view(torch.complex128)])) == 2
    assert _contiguous_runs([]) == []
