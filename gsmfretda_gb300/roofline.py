"""ALU cost model of the photon-burst Monte-Carlo PDA, evaluated on a workload.

The path has no dense contraction and reads a few bytes per unit, so its
roofline is the FP32/INT32 lane-operation rate (152 SMs x 128 lanes x SM
clock). The algorithmic work of one unit (parameter set, burst, MC sample) is
counted with fixed costs per operation:

    PHILOX_WORD     25  INT32 ops per 32-bit Philox4x32-10 word (~100 per block)
    LOG             16  FP32 ops per logarithm (one per dwell)
    BINOMIAL        40  ops per binomial draw (BTRD, or a table inversion)
    SEARCH_STEP      4  ops per bisection step over a burst's sorted arrival
                        offsets (midpoint, load, compare, select)
    EXP             16  FP32 ops per exponential (e^-lam of a Poisson inversion)
    POISSON_STEP     4  ops per step of the Poisson inversion (compare,
                        subtract, two multiplies)
    SPLIT_TRIAL      3  ops per background photon split into acceptor/donor

and the draws of the photon-by-photon model: with D dwell segments per unit,
1 + 2D + 4 + D random words (initial state; jump and dwell per segment;
background; one binomial per segment), D logarithms and D binomials, one
bisection of the burst's N sorted offsets per segment that ends inside the
burst (the last segment takes the photons left), and the segment's Poisson
background pair: an exponential, T + 1 inversion steps for a count T, and T
split trials, where the counts of a unit's segments add up to lam_B = (bg_a +
bg_d) T on average over a burst of duration T:

    ops(D, N) = PHILOX_WORD (5 + 3 D) + (LOG + BINOMIAL) D
                + SEARCH_STEP (D - 1) log2(N + 1)
                + EXP D + POISSON_STEP (lam_B + D) + SPLIT_TRIAL lam_B.

A linear scan that compares every photon once (PHOTON_COMPARE = 2 ops per
photon, 2 N per unit) is the other way to assign photons; it is reported
beside the model for comparison, not counted: the kernels bisect.

D is computed from the workload, not assumed: a trajectory started from the
stationary law pi of the rate matrix K jumps at the stationary flux
sum_s pi_s k_exit(s), so over a burst of duration T it has on average
1 + T sum_s pi_s k_exit(s) segments (exact for the model's stationary start).
"""
import numpy as np

PHILOX_WORD = 25
LOG = 16
BINOMIAL = 40
SEARCH_STEP = 4
EXP = 16
POISSON_STEP = 4
SPLIT_TRIAL = 3
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


def photon_ops_breakdown(n, args, N, T, bg=0.0):
    """The cost model's terms per unit on bursts with photon counts N and
    durations T, background rate bg = bg_a + bg_d (per second): draws (Philox
    words, logarithms, binomials), search (the bisections that assign photons
    to segments), background (the segments' Poisson pairs), their sum, the
    linear-scan alternative (not counted), D and lam_B."""
    D = mean_segments(n, args, T)
    Nbar = float(np.mean(np.asarray(N, dtype=np.float64)))
    lam = float(bg) * float(np.mean(np.asarray(T, dtype=np.float64)))
    draws = PHILOX_WORD * (5.0 + 3.0 * D) + (LOG + BINOMIAL) * D
    search = SEARCH_STEP * (D - 1.0) * float(np.log2(Nbar + 1.0))
    background = EXP * D + POISSON_STEP * (lam + D) + SPLIT_TRIAL * lam if bg > 0.0 else 0.0
    return {"draws": draws, "search": search, "background": background,
            "ops": draws + search + background, "linear_scan": PHOTON_COMPARE * Nbar,
            "segments": D, "mean_photons": Nbar, "background_photons": lam}


def photon_ops_per_unit(n, args, N, T, bg=0.0):
    """(ops per unit, D) of the photon-by-photon model on bursts with photon
    counts N and durations T and background rate bg."""
    b = photon_ops_breakdown(n, args, N, T, bg)
    return b["ops"], b["segments"]


def lane_peak_gops(sm_mhz, sms=152, lanes=128):
    """FP32/INT32 lane operations per second of the GPU, in Gop/s."""
    return sms * lanes * sm_mhz * 1e6 / 1e9
