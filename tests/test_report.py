"""The native report writers (fame_report_*) against the reference's own
writers: printMethylationLevels (ReadQueue.cpp:1860-1893) and the single-cell
matrix (the single-cell ReadQueue's header, ReadQueue.cpp:182-215, and
printSCMethylationLevels, 1894-1921), run by the compiled reference
(oracle/_ref) on the same index tables and tallies, byte for byte.  Where
the reference library is not built, the expected text is formatted here."""
import numpy as np
import pytest

from fame_gb300 import SingleCellQueue, write_cpg_report


@pytest.fixture(scope="module")
def ref_index(product_index):
    try:
        from oracle import refbind
        if not refbind.available():
            return None
        L = refbind.RefLib()
        t = product_index.tables(sparse=False)

        class A:
            pass

        a = A()
        a.chrom_seqs = product_index.chrom_seqs()
        a.chrom_names = product_index.chrom_names()
        for k, v in t.items():
            setattr(a, k, v)
        a.tab_index64 = product_index.tab_index64
        return L.from_arrays(a)
    except OSError:
        return None


def expected_cpg(index, meth):
    t = index.tables()
    names = index.chrom_names()
    lines = []
    for i, (c, p) in enumerate(zip(t["cpg_chrom"], t["cpg_pos"].astype(np.int64))):
        m = meth[i]
        lines.append("%s\t%d\t%d\t%d\t%d\t%d\n" % (names[c], (p + index.readlen - 2) & 0xFFFFFFFF, m[0], m[1], m[2], m[3]))
    return "".join(lines)


def test_cpg_report_matches_reference(product_index, ref_index, tmp_path):
    rng = np.random.default_rng(9)
    meth = rng.integers(0, 65536, size=(product_index.n_cpg, 4)).astype(np.uint16)
    meth[: product_index.n_cpg // 3] = 0
    out = tmp_path / "r_cpg.tsv"
    write_cpg_report(str(out), product_index, meth, n_threads=3)
    if ref_index is not None:
        exp = open(ref_index.print_cpg(meth, str(tmp_path / "ref")), "rb").read()
        assert out.read_bytes() == exp
    else:
        assert out.read_text() == expected_cpg(product_index, meth)


class _FakeGpu:
    def __init__(self, rows):
        self.rows = list(rows)

    def tallies(self, reset=False):
        return self.rows.pop(0)


def test_single_cell_matrix_matches_reference(product_index, ref_index, tmp_path):
    rng = np.random.default_rng(10)
    n = product_index.n_cpg
    cells = [("cellA", rng.integers(0, 900, size=(n, 4)).astype(np.uint16)),
             ("cellB", rng.integers(0, 3, size=(n, 4)).astype(np.uint16))]
    out = tmp_path / "sc.tsv"
    sc = SingleCellQueue(str(out), product_index, _FakeGpu([m for _, m in cells]))
    for cid, _ in cells:
        sc.print_sc_methylation_levels(cid)
    sc.close()
    if ref_index is not None:
        ref_path = str(tmp_path / "ref_sc.tsv")
        ref_index.print_sc(ref_path, cells)
        assert out.read_bytes() == open(ref_path, "rb").read()
        return
    t = product_index.tables(sparse=False)
    names = product_index.chrom_names()
    exp = "\nSC_ID\tCount_Type\t" + "".join("%s\t" % names[c] for c in t["cpg_chrom"])
    exp += "\nSC_ID\tCount_Type\t" + "".join("%d\t" % (p + product_index.readlen - 2)
                                            for p in t["cpg_pos"].astype(np.int64))
    for cid, m in cells:
        for col, label in ((0, "methFwd"), (1, "unmethFwd"), (2, "methRev"), (3, "unmethFwd")):
            exp += "\n%s\t%s\t" % (cid, label) + "".join("%d\t" % v for v in m[:, col])
    assert out.read_text() == exp
