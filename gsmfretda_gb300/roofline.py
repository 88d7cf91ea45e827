"""ALU cost model of the photon-burst Monte-Carlo PDA, evaluated on a workload.

The path has no dense contraction and reads a few bytes per unit, so its
roofline is the FP32/INT32 lane-operation rate (152 SMs x 128 lanes x SM
clock). The algorithmic work of one unit (parameter set, burst, MC sample) is
counted with fixed costs per operation:

    PHILOX_WORD     25  INT32 ops per 32-bit Philox4x32-10 word (~100 per block)
    LOG             16  FP32 ops per logarithm (one per dwell)
    BINOMIAL        40  ops per binomial draw (BTRD, or a table inversion)
    PHOTON_COMPARE   2  ops per photon assigned to a segment (photon mode)

and the draws of the photon-by-photon model: with D dwell segments per unit,
1 + 2D + 4 + D random words (initial state; jump and dwell per segment;
background; one binomial per segment), D logarithms and D binomials, and every
photon compared once:

    ops(D, N) = PHILOX_WORD (5 + 3 D) + (LOG + BINOMIAL) D + PHOTON_COMPARE N.

D is computed from the workload, not assumed: a trajectory started from the
stationary law pi of the rate matrix K jumps at the stationary flux
sum_s pi_s k_exit(s), so over a burst of duration T it has on average
1 + T sum_s pi_s k_exit(s) segments (exact for the model's stationary start).
"""
import numpy as np

PHILOX_WORD = 25
LOG = 16
BINOMIAL = 40
PHOTON_COMPARE = 2


def rate_matrix(n, args):
    """K (K[i, j] = rate j -> i) from the reference parameter vector
    [E(n), K off-diagonals row-major without the diagonal, V(n)]
    (src/mc.cu:792-800), in float64."""
    a = np.asarray(args, dtype=np.float64).reshape(-1)
    K = np.zeros((n, n))
    koff = a[n:n + n * (n - 1)]
    k = 0
    for i in range(n):
        for j in range(n):
            if i != j:
                K[i, j] = koff[k]
                k += 1
    return K


def stationary(K):
    """pi with (K - diag(k_exit)) pi = 0, sum(pi) = 1 (least squares, float64)."""
    n = K.shape[0]
    Q = K - np.diag(K.sum(axis=0))
    A = np.vstack([Q, np.ones(n)])
    b = np.zeros(n + 1)
    b[-1] = 1.0
    return np.linalg.lstsq(A, b, rcond=None)[0]


def mean_segments(n, args, T):
    """Expected dwell segments per unit over bursts of durations T."""
    K = rate_matrix(n, args)
    flux = float(stationary(K) @ K.sum(axis=0))
    return 1.0 + flux * float(np.mean(np.asarray(T, dtype=np.float64)))


def photon_ops_per_unit(n, args, N, T):
    """(ops per unit, D) of the photon-by-photon model on bursts with photon
    counts N and durations T."""
    D = mean_segments(n, args, T)
    Nbar = float(np.mean(np.asarray(N, dtype=np.float64)))
    ops = PHILOX_WORD * (5.0 + 3.0 * D) + (LOG + BINOMIAL) * D + PHOTON_COMPARE * Nbar
    return ops, D


def lane_peak_gops(sm_mhz, sms=152, lanes=128):
    """FP32/INT32 lane operations per second of the GPU, in Gop/s."""
    return sms * lanes * sm_mhz * 1e6 / 1e9
