"""Parameter-vector layout and derived tables (host-only; no GPU).

Restates the reference's CPU test (tests/ParamsTest.cpp:26-72, n = 2..6):
column-major K, P_i2j columns summing to 1 within 1e-5, and for n = 3 the
ratio consistency P(i,j)/P(ii,j) == K(i,j)/K(ii,j) within 1e-4. Checks that
the product's host derivation (gpda_build_params) and the oracle's are the
same bits, and that the stationary distribution solves K pi = 0."""
import numpy as np
import pytest

from gsmfretda_gb300.synth import pack_args, unpack_args

# DevParams layout in floats (include/gpda.h, gpda_internal.h)
OFF = dict(n=0, anyV=1, E=4, V=12, eps=20, kexit=28, inv_kexit=36, init_cdf=44, jump_cdf=52,
           K=116, Pi2j=180, pinit=244)


def rand_args(n, seed):
    """MatCheck::genRandMatk (tests/ParamsTest.cpp:10-24): E~U(0,1), K~U(0,1000), V~U(0,10)."""
    rs = np.random.RandomState(seed)
    return np.concatenate([rs.uniform(0, 1, n), rs.uniform(0, 1000, n * (n - 1)),
                           rs.uniform(0, 10, n)]).astype(np.float32)


def product_tables(n, args):
    from gsmfretda_gb300.api import build_params
    f = build_params(n, args)
    K = f[OFF["K"]:OFF["K"] + n * n].reshape(n, n).T          # [row i, col j]
    P = f[OFF["Pi2j"]:OFF["Pi2j"] + n * n].reshape(n, n).T
    return f, K, P


@pytest.mark.parametrize("n", [2, 3, 4, 5, 6])
def test_reference_param_invariants(gpda_lib, n):
    args = rand_args(n, 100 + n)
    f, K, P = product_tables(n, args)
    _, Kin, _ = unpack_args(args, n)
    for i in range(n):
        for j in range(n):
            if i != j:
                assert K[i, j] == np.float32(Kin[i, j])       # K(i,j) = rate j -> i
    # column-major: matKmp(0,i) == matK[i*n]
    flat = f[OFF["K"]:OFF["K"] + n * n]
    for i in range(n):
        assert K[0, i] == flat[i * n]
    for j in range(n):
        assert abs(P[:, j].sum() - 1.0) < 1e-5
        assert abs(K[:, j].sum()) < 1e-3 * np.abs(K[:, j]).max()   # diag = -column sum
        if n == 3:
            i, ii = (j + 1) % n, (j + 2) % n
            assert abs(P[i, j] / P[ii, j] - K[i, j] / K[ii, j]) < 1e-4


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 6, 7, 8])
def test_product_and_oracle_tables_identical(gpda_lib, orc, n):
    args = rand_args(n, 200 + n)
    m = orc.model()
    f, _, _ = product_tables(n, args)
    o = np.frombuffer(bytes(orc.build_params(n, args, m)), dtype=np.float32)
    f = f[:o.size]                      # the product appends precomputed binomial constants
    mask = np.ones(o.size, dtype=bool)
    mask[OFF["anyV"]] = False           # product-only flag word
    np.testing.assert_array_equal(f.view(np.uint32)[mask], o.view(np.uint32)[mask])


@pytest.mark.parametrize("n", [2, 3, 4, 6, 8])
def test_stationary_distribution(gpda_lib, n):
    args = rand_args(n, 300 + n)
    f, K, _ = product_tables(n, args)
    cdf = f[OFF["init_cdf"]:OFF["init_cdf"] + n].astype(np.float64)
    pi = np.diff(np.concatenate([[0.0], cdf]))
    assert abs(cdf[-1] - 1.0) < 1e-6
    assert np.abs(K.astype(np.float64) @ pi).max() < 1e-4 * np.abs(K).max()


def test_precomputed_binomial_constants(gpda_lib, orc):
    n = 5
    args = rand_args(n, 9)
    f, _, _ = product_tables(n, args)
    eps = f[OFF["eps"]:OFF["eps"] + n]
    pp = f[252:252 + n]
    logq = f[260:260 + n]
    rr = f[268:268 + n]
    L = orc.lib()
    for i in range(n):
        want_pp = np.float32(1.0) - eps[i] if eps[i] > 0.5 else eps[i]
        q = np.float32(1.0) - want_pp
        assert pp[i] == want_pp
        assert logq[i] == np.float32(L.orc_logf(float(q)))   # same FP32 log on both sides
        assert rr[i] == np.float32(want_pp / q)


def test_exit_rates_and_jump_cdf(gpda_lib):
    n = 4
    args = rand_args(n, 7)
    f, K, P = product_tables(n, args)
    kexit = f[OFF["kexit"]:OFF["kexit"] + n]
    np.testing.assert_allclose(kexit, -np.diag(K), rtol=1e-6)
    jc = f[OFF["jump_cdf"]:OFF["jump_cdf"] + 64].reshape(8, 8)
    for j in range(n):
        probs = np.diff(np.concatenate([[0.0], jc[j, :n]]))
        np.testing.assert_allclose(probs, P[:, j], atol=2e-6)


def test_eps_formula(gpda_lib):
    from gsmfretda_gb300.api import build_params
    args = pack_args([0.0, 0.3, 1.0], np.full((3, 3), 100.0) - np.eye(3) * 100.0)
    f = build_params(3, args, gamma=0.8, crosstalk=0.05)
    E = np.array([0.0, 0.3, 1.0])
    eps = (0.8 * E + 0.05 * (1 - E)) / (0.8 * E + 1.05 * (1 - E))
    np.testing.assert_allclose(f[OFF["eps"]:OFF["eps"] + 3], eps, rtol=1e-6)


def test_invalid_parameters_rejected(gpda_lib):
    from gsmfretda_gb300._lib import GpdaError
    from gsmfretda_gb300.api import build_params
    good = rand_args(3, 1)
    for bad_idx, val in [(0, 1.5), (0, -0.1), (5, -1.0), (10, np.inf), (11, np.nan)]:
        a = good.copy()
        a[bad_idx] = val
        with pytest.raises(GpdaError) as e:
            build_params(3, a)
        assert e.value.code == -1
    # disconnected chain: no unique stationary distribution
    K = np.zeros((3, 3))
    K[1, 0] = 5.0
    with pytest.raises(GpdaError) as e:
        build_params(3, pack_args([0.1, 0.5, 0.9], K))
    assert e.value.code == -2
    with pytest.raises(GpdaError):
        build_params(9, np.zeros(90, dtype=np.float32))


def test_pack_unpack_roundtrip():
    rs = np.random.RandomState(3)
    for n in range(1, 9):
        E = rs.uniform(0, 1, n)
        K = rs.uniform(0, 100, (n, n))
        np.fill_diagonal(K, 0)
        V = rs.uniform(0, 2, n)
        a = pack_args(E, K, V)
        assert a.size == n * (n + 1)
        E2, K2, V2 = unpack_args(a, n)
        np.testing.assert_allclose(E2, E.astype(np.float32))
        np.testing.assert_allclose(K2, K.astype(np.float32))
        np.testing.assert_allclose(V2, V.astype(np.float32))
