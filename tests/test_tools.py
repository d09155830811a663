"""The file tools around the product, against the reference's own programs
compiled from its sources (aurora.x, mars.x, vulcan.x) where the reference
tree is present, and against the generator's files everywhere.  Host only."""
import filecmp
import os

import numpy as np
import pytest

import jupiterncsm_gb300 as jn
import oracle


def rows(path):
    return sorted(l.strip() for l in open(path) if l.startswith("BLOCK:"))


@pytest.fixture(scope="module")
def he4(tmp_path_factory):
    """He4 Nmax 4, two- plus three-body, with the lists also in Anicre's raw and text forms."""
    root = tmp_path_factory.mktemp("tools")
    raw, text = str(root / "raw"), str(root / "text")
    jn.generate(raw, Z=2, N=2, nmax=4, nbody=3, basis_files=False, anicre_lists=1)
    jn.generate(text, Z=2, N=2, nmax=4, nbody=3, basis_files=False, anicre_lists=2)
    return root, raw, text


def list_files(d):
    return sorted(f for f in os.listdir(d) if f.startswith("index_list_"))


@pytest.mark.parametrize("human_readable", [False, True])
def test_aurora_rebuilds_the_index_lists(he4, human_readable):
    root, raw, text = he4
    src = text if human_readable else raw
    out = str(root / f"aurora_{int(human_readable)}")
    n = jn.aurora(f"{src}/comb.txt", f"{src}/anicr_lists", out, 2, 2, human_readable=human_readable)
    want = list_files(f"{src}/index_lists")
    assert n == len(want) and list_files(out) == want
    for f in want:
        assert filecmp.cmp(f"{out}/{f}", f"{src}/index_lists/{f}", shallow=False), f
    if oracle.reference_tool_available("aurora"):
        ref = str(root / f"ref_aurora_{int(human_readable)}")
        os.makedirs(ref)
        args = ["--human-readable"] if human_readable else []
        assert oracle.reference_tool("aurora", f"{src}/comb.txt", f"{src}/anicr_lists", ref, 2, 2, *args).returncode == 0
        assert list_files(ref) == want
        for f in want:
            assert filecmp.cmp(f"{out}/{f}", f"{ref}/{f}", shallow=False), f


def test_aurora_skips_three_body_lists_and_missing_files(he4, capfd):
    root, raw, _ = he4
    out = str(root / "aurora_no3")
    n = jn.aurora(f"{raw}/comb.txt", f"{raw}/anicr_lists", out, 2, 2, skip_three_body=True)
    three = [l for l in open(f"{raw}/comb.txt") if "ARRAY:" in l and l.split()[0] in ("ppp", "nnn", "nnp", "npp")]
    assert n == len(list_files(f"{raw}/index_lists")) - len(three) > 0
    # a list Anicre did not write is reported and skipped, as aurora.x does
    victim = sorted(os.listdir(f"{raw}/anicr_lists/p_inds_index_lists"))[0]
    os.rename(f"{raw}/anicr_lists/p_inds_index_lists/{victim}", f"{root}/{victim}")
    try:
        m = jn.aurora(f"{raw}/comb.txt", f"{raw}/anicr_lists", str(root / "aurora_missing"), 2, 2)
    finally:
        os.rename(f"{root}/{victim}", f"{raw}/anicr_lists/p_inds_index_lists/{victim}")
    assert m == len(list_files(f"{raw}/index_lists")) - 1
    assert "Could not open file" in capfd.readouterr().err


def test_aurora_empty_anicre_list(tmp_path):
    """An Anicre list with no entries becomes an empty index_list_<id>, as with
    aurora.x (byte for byte, where the reference tool is built)."""
    import shutil
    raw = str(tmp_path / "raw")
    jn.generate(raw, Z=2, N=2, nmax=2, nbody=3, basis_files=False, anicre_lists=1)
    d0 = f"{raw}/anicr_lists/n_inds_index_lists"
    open(f"{d0}/{sorted(os.listdir(d0))[0]}", "wb").close()
    out = str(tmp_path / "ours")
    n = jn.aurora(f"{raw}/comb.txt", f"{raw}/anicr_lists", out, 2, 2)
    assert n == len(list_files(f"{raw}/index_lists"))
    empty = [f for f in list_files(out) if os.path.getsize(f"{out}/{f}") == 0]
    assert len(empty) == 1
    if oracle.reference_tool_available("aurora"):
        ref = str(tmp_path / "ref")
        os.makedirs(ref)
        assert oracle.reference_tool("aurora", f"{raw}/comb.txt", f"{raw}/anicr_lists", ref, 2, 2).returncode == 0
        assert list_files(ref) == list_files(out)
        for f in list_files(out):
            assert filecmp.cmp(f"{out}/{f}", f"{ref}/{f}", shallow=False), f
    shutil.rmtree(raw)


@pytest.mark.parametrize("two_body_only", [False, True])
def test_mars_writes_the_reference_instruction_set(he4, two_body_only):
    root, raw, _ = he4
    out = str(root / f"order_{int(two_body_only)}.txt")
    n = jn.mars(f"{raw}/comb.txt", 2, 2, out, two_body_only=two_body_only)
    got = rows(out)
    assert len(got) == n > 0
    if not two_body_only:
        assert got == rows(f"{raw}/evaluation_order.txt")
    if oracle.reference_tool_available("mars"):
        ref = str(root / f"ref_order_{int(two_body_only)}.txt")
        args = ["--only-two-nucleon-forces"] if two_body_only else []
        assert oracle.reference_tool("mars", f"{raw}/comb.txt", ref, "--num-protons", 2, "--num-neutrons", 2,
                                     *args).returncode == 0
        assert got == rows(ref)


def test_mars_order_gives_the_same_product(he4):
    """The reference kernels applied in the exported order give the original product."""
    root, raw, _ = he4
    order = str(root / "order_product.txt")
    jn.mars(f"{raw}/comb.txt", 2, 2, order)
    P = oracle.Port(raw)
    x = np.random.default_rng(3).standard_normal(P.dimension)
    want = P.matvec(x)
    Q = oracle.Port(raw, order=order)
    got = Q.matvec(x)
    assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()


def test_vulcan_sums_operators(he4, tmp_path):
    root, raw, _ = he4
    other = str(root / "other")
    jn.generate(other, Z=2, N=2, nmax=4, nbody=3, seed=99, hbar_omega=0.0, basis_files=False, me_only_subdir="me")
    ops = [(f"{raw}/matrix_elements", 0.75), (f"{other}/me", -1.5)]
    out = str(tmp_path / "sum")
    jn.vulcan(f"{raw}/comb.txt", 2, 2, ops, out)
    files = sorted(f for f in os.listdir(f"{raw}/matrix_elements"))
    assert files and sorted(os.listdir(out)) == files
    for f in files[:50]:
        a, b, s = (oracle.read_me_file(f"{d}/{f}") for d in (ops[0][0], ops[1][0], out))
        assert s[:2] == a[:2] and np.array_equal(s[2], 0.75 * a[2] + (-1.5) * b[2])
    if oracle.reference_tool_available("vulcan"):
        ref = str(tmp_path / "ref_sum")
        os.makedirs(ref)
        assert oracle.reference_tool("vulcan", ref, f"{raw}/comb.txt", 2, 2, ops[0][0], "-c", 0.75, ops[1][0], "-c",
                                     -1.5).returncode == 0
        for f in files:
            assert filecmp.cmp(f"{out}/{f}", f"{ref}/{f}", shallow=False), f
