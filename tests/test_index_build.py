"""The product's host index builder (fame_index_build) against the oracle and
the reference's tables."""
import hashlib

import numpy as np


def _digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_product_build_matches_oracle(product_index, oracle_index):
    t = product_index.tables()
    for k, v in oracle_index.t.items():
        assert np.array_equal(t[k], v), k


def test_product_build_matches_reference(golden, product_index):
    dig = golden["digests"].item()
    t = product_index.tables()
    for k in ("cpg_pos", "bucket_key", "bucket_start", "kmer_meta", "strand", "win_sind", "win_eind"):
        assert _digest(t[k]) == dig[k], k
    assert product_index.readlen == 100
    seqs = product_index.chrom_seqs()
    assert [len(s) for s in seqs] == list(golden["chrom_lens"])


def test_build_rejects_bad_arguments():
    from fame_gb300 import FameError, HostIndex
    import pytest
    with pytest.raises(FameError):
        HostIndex.build([], readlen=100)
    with pytest.raises(FameError):
        HostIndex.build([b"ACGT" * 100], readlen=20)
    # the device build checks its arguments before touching a GPU
    with pytest.raises(FameError):
        HostIndex.build_gpu([], readlen=100)
    with pytest.raises(FameError):
        HostIndex.build_gpu([b"ACGT" * 100], readlen=4096)
