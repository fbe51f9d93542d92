"""CPU: host-side logic of the lineax-style API (dispatch, structures, result
codes, ragged layout) — nothing here launches a kernel."""

import pytest
import torch

import lineax_gb300 as lx
from lineax_gb300 import batched
from lineax_gb300._structure import ravel, structure_of, tree_flatten, tree_unflatten, unravel


def test_results_codes_match_lineax_order():
    names = ["successful", "max_steps_reached", "singular", "breakdown", "stagnation",
             "conlim", "nonfinite_input"]
    for i, name in enumerate(names):
        assert getattr(lx.RESULTS, name) == i
        assert lx.RESULTS.name(i) == name
    assert lx.RESULTS[lx.RESULTS.successful] == ""


def _mat(tags=(), n=3):
    return lx.MatrixLinearOperator(torch.eye(n, dtype=torch.float64), tags)


@pytest.mark.parametrize(
    "tags,expected",
    [
        ((), lx.LU),
        (lx.lower_triangular_tag, lx.Triangular),
        (lx.upper_triangular_tag, lx.Triangular),
        (lx.positive_semidefinite_tag, lx.Cholesky),
        (lx.negative_semidefinite_tag, lx.Cholesky),
        (lx.diagonal_tag, lx.Diagonal),
    ],
)
def test_auto_solver_dispatch_well_posed(tags, expected):
    s = lx.AutoLinearSolver(well_posed=True).select_solver(_mat(tags))
    assert isinstance(s, expected)


def test_auto_solver_nonsquare():
    op = lx.MatrixLinearOperator(torch.zeros(5, 3, dtype=torch.float64))
    assert isinstance(lx.AutoLinearSolver(well_posed=None).select_solver(op), lx.QR)
    with pytest.raises(ValueError):
        lx.AutoLinearSolver(well_posed=True).select_solver(op)


def test_transpose_tags():
    t = lx.transpose_tags(frozenset([lx.lower_triangular_tag, lx.unit_diagonal_tag]))
    assert t == frozenset([lx.upper_triangular_tag, lx.unit_diagonal_tag])
    sym = frozenset([lx.symmetric_tag, lx.lower_triangular_tag])
    assert lx.transpose_tags(sym) == sym


def test_raw_array_rejected():
    with pytest.raises(ValueError):
        lx.linear_solve(torch.eye(2), torch.ones(2))


def test_structure_mismatch_rejected():
    op = _mat(n=3)
    with pytest.raises(ValueError):
        lx.linear_solve(op, torch.ones(4, dtype=torch.float64))


def test_solver_init_checks():
    with pytest.raises(ValueError):
        lx.Cholesky().init(_mat(), {})
    with pytest.raises(ValueError):
        lx.Triangular().init(_mat(), {})
    with pytest.raises(ValueError):
        lx.LU().init(lx.MatrixLinearOperator(torch.zeros(2, 3, dtype=torch.float64)), {})


def test_pytree_ravel_roundtrip():
    tree = {"b": torch.arange(3.0), "a": (torch.tensor(1.0), torch.arange(4.0).reshape(2, 2))}
    leaves, td = tree_flatten(tree)
    assert [tuple(x.shape) for x in leaves] == [(), (2, 2), (3,)]  # sorted dict keys
    flat = ravel(tree, torch.float64)
    assert flat.tolist() == [1.0, 0, 1, 2, 3, 0, 1, 2]
    back = unravel(flat, structure_of(tree))
    assert torch.equal(back["b"], tree["b"].double())
    assert tree_unflatten(td, leaves)["a"][0] is leaves[0]


def test_ragged_layout_offsets():
    a_off, b_off, ta, tb = batched.RaggedBatch.layout([2, 3], [1, 2])
    assert a_off == [0, 4] and b_off == [0, 2] and ta == 13 and tb == 8


def test_identity_operator_short_circuit():
    op = lx.IdentityLinearOperator(torch.zeros(3, dtype=torch.float64))
    v = torch.arange(3.0, dtype=torch.float64)
    sol = lx.linear_solve(op, v)
    assert sol.value is v and sol.result == lx.RESULTS.successful


def test_complex_real_forms():
    """Complex problems are solved through real forms (lineax_gb300._complex):
    R(A) [Re x; Im x] = [Re Ax; Im Ax], Hermitian definiteness maps to
    symmetric definiteness, and the diagonal-scaled interleaved form of a
    triangular matrix is unit triangular with the same solution."""
    import pytest
    import torch

    import lineax_gb300 as lx
    from lineax_gb300 import _complex

    g = torch.Generator().manual_seed(3)
    a = torch.randn(5, 4, dtype=torch.complex128, generator=g)
    x = torch.randn(4, dtype=torch.complex128, generator=g)
    r = _complex.real_form_matrix(a)
    assert r.dtype == torch.float64 and r.shape == (10, 8)
    assert torch.allclose(r @ _complex.to_real(x), _complex.to_real(a @ x))
    assert torch.allclose(_complex.from_real(_complex.to_real(x)), x)
    # Hermitian positive definite A: R(A) symmetric positive definite
    h = a.conj().T @ a + torch.eye(4, dtype=torch.complex128)
    rh = _complex.real_form_matrix(h)
    assert torch.allclose(rh, rh.T) and bool((torch.linalg.eigvalsh(rh) > 0).all())
    tags = _complex.real_form_tags({lx.positive_semidefinite_tag})
    assert tags == {lx.positive_semidefinite_tag, lx.symmetric_tag}
    assert _complex.real_form_tags({lx.symmetric_tag, lx.lower_triangular_tag}) == frozenset()
    # complex PSD means Hermitian, not symmetric (lineax/_operator.py:1617-1631)
    assert not lx.is_symmetric(lx.MatrixLinearOperator(h, lx.positive_semidefinite_tag))
    assert lx.is_symmetric(lx.MatrixLinearOperator(h.real, lx.positive_semidefinite_tag))
    # triangular: D^-1 T in interleaved real form is unit lower triangular
    t = torch.tril(torch.randn(4, 4, dtype=torch.complex128, generator=g)) + 3 * torch.eye(4)
    d = torch.diagonal(t)
    ts = t / d[:, None]
    e = torch.zeros(8, 8, dtype=torch.float64)
    e[0::2, 0::2], e[0::2, 1::2] = ts.real, -ts.imag
    e[1::2, 0::2], e[1::2, 1::2] = ts.imag, ts.real
    assert torch.allclose(torch.triu(e, 1), torch.zeros_like(e), atol=1e-15)
    assert torch.allclose(torch.diagonal(e), torch.ones(8, dtype=torch.float64))
    xt = torch.randn(4, dtype=torch.complex128, generator=g)
    inter = torch.stack([xt.real, xt.imag], 1).reshape(-1)
    rhs = (t @ xt) / d
    assert torch.allclose(e @ inter, torch.stack([rhs.real, rhs.imag], 1).reshape(-1))
    # a complex vector for a real operator is a structure mismatch, as in lineax
    op = lx.MatrixLinearOperator(torch.eye(3, dtype=torch.float64))
    with pytest.raises(ValueError, match="structures do not match"):
        lx.linear_solve(op, torch.ones(3, dtype=torch.complex128), lx.LU())


def test_host_solver_chunk_bounds():
    from lineax_gb300.batched import chunk_bounds

    assert chunk_bounds([5, 5, 5, 5], 2) == [0, 2, 4]
    assert chunk_bounds([5, 5, 5, 5], 1) == [0, 4]
    assert chunk_bounds([5, 5], 8) == [0, 1, 2]          # at most one range per system
    assert chunk_bounds([100, 1, 1, 1], 2) == [0, 1, 4]   # the large system closes a range
    assert chunk_bounds([1] * 10, 3) == [0, 4, 7, 10]
    b = chunk_bounds([3, 0, 7, 2, 9, 4, 4, 1], 4)
    assert b[0] == 0 and b[-1] == 8 and all(x < y for x, y in zip(b, b[1:]))
