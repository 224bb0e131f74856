"""Initial crack on the host: the restatement against the reference's own
compiled ``create_crack`` (``peripy/create_crack.pyx:1-43``), and the
argument checks of the GPU entry point that run before any CUDA call.

The GPU path itself is compared in ``test_gpu_crack.py``.
"""
import numpy as np
import pytest

from tests.crack_cases import crack_cases


@pytest.fixture(scope="module")
def ref_crack():
    from oracle import build_ref
    if not build_ref.available():
        build_ref.build(quiet=True)
    if not build_ref.available():
        pytest.skip("reference checkout absent and no generated C")
    return build_ref.load("create_crack").create_crack


@pytest.mark.parametrize("case", range(6))
def test_restatement_matches_reference(case, ref_crack):
    from probabilistic_peridynamics_gb300.model import create_crack
    crack, nlist, n_neigh = crack_cases(case)
    want_nl, want_nn = nlist.copy(), n_neigh.copy()
    ref_crack(crack, want_nl, want_nn)
    got_nl, got_nn = nlist.copy(), n_neigh.copy()
    create_crack(crack, got_nl, got_nn)
    assert np.array_equal(got_nl, want_nl)
    assert np.array_equal(got_nn, want_nn)
    assert not np.array_equal(want_nn, n_neigh)  # the case cuts something


def test_reference_raises_after_applying_earlier_pairs(ref_crack):
    """The behaviour the GPU wrapper mirrors on a bad index."""
    crack, nlist, n_neigh = crack_cases(0)
    bad = crack.copy()
    bad[5] = (nlist.shape[0], 0)
    want_nl, want_nn = nlist.copy(), n_neigh.copy()
    ref_crack(crack[:5].copy(), want_nl, want_nn)
    nl, nn = nlist.copy(), n_neigh.copy()
    with pytest.raises(IndexError):
        ref_crack(bad, nl, nn)
    assert np.array_equal(nl, want_nl) and np.array_equal(nn, want_nn)


def test_gpu_wrapper_checks_before_any_cuda_call():
    from probabilistic_peridynamics_gb300.neighbours import create_crack
    _, nlist, n_neigh = crack_cases(0)
    with pytest.raises(TypeError):
        create_crack([[0, 1]], nlist.astype(np.int64), n_neigh)
    with pytest.raises(TypeError):
        create_crack([[0, 1]], np.asfortranarray(nlist), n_neigh)
    with pytest.raises(ValueError):
        create_crack([[0, 1]], nlist, n_neigh[:-1].copy())
    # the first pair is out of range: nothing to apply, IndexError at once
    nl, nn = nlist.copy(), n_neigh.copy()
    with pytest.raises(IndexError):
        create_crack([[nlist.shape[0], 0], [0, 1]], nl, nn)
    assert np.array_equal(nl, nlist) and np.array_equal(nn, n_neigh)
    # an empty crack list changes nothing and needs no GPU
    create_crack(np.zeros((0, 2), dtype=np.int32), nl, nn)
    assert np.array_equal(nl, nlist)
