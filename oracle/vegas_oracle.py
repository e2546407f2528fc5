"""NumPy float64 restatement of vegasflow's VEGAS hot path -- TEST INFRASTRUCTURE ONLY.

Never imported by the product package.  Each function names the reference
location (path within N3PDF/vegasflow 1.4.0) whose arithmetic it restates.  The
element-wise operations are written in the same order as the reference's
TensorFlow graph, as separate IEEE-754 float64 operations (no fused
multiply-add), so that bin indices, sampled points and weights are bit-exact
against the reference on identical uniforms.  Reductions (sums over events,
the 50-bin sums of the refinement) use NumPy's order; their results agree with
the reference to rounding level.

The Philox4x32-10 generator below is *this project's* counter-based stream
(Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3",
SC'11), restated from the published algorithm so the GPU's in-kernel stream can
be checked event by event.  The reference draws its uniforms from TensorFlow's
generator, which cannot be reproduced here; parity against the reference itself
is therefore established on injected uniforms.
"""

from __future__ import annotations

import math
from concurrent.futures import ThreadPoolExecutor
from itertools import product

import numpy as np

__all__ = [
    "BINS_MAX", "ALPHA", "BETA", "TECH_CUT", "MAX_EVENTS_LIMIT", "MAX_NEVAL_HCUBE",
    "philox4x32_10", "philox_words", "uniforms_f64_philox", "tech_cut_affine",
    "words_to_u53", "vegas_map", "plus_map", "importance_sampling_digest",
    "consume_array_into_indices", "refine_grid_per_dimension", "refine_grid",
    "initial_grid", "plus_stratification", "redistribute_samples",
    "weighted_average", "chunk_sizes", "vegas_map_f32_words", "f32_weight_prescale", "plain_map_f32_words",
    "OracleVegas", "OraclePlain", "OraclePlus", "INTEGRANDS", "integrand_symgauss",
    "integrand_gauss_mu", "integrand_breit_wigner", "integrand_prod", "integrand_sum",
    "symgauss_exact", "gauss_mu_exact", "breit_wigner_exact", "threaded_vegas_iteration",
    "uniforms_of_words", "plus_bins_from_words", "plus_map_f32_words", "hypercube_points",
    "fma_f32",
]

# configflow.py:13-24
BINS_MAX = 50
ALPHA = 1.5
BETA = 0.75
TECH_CUT = 1e-8
MAX_EVENTS_LIMIT = int(1e6)
MAX_NEVAL_HCUBE = int(1e4)

_MASK32 = np.uint64(0xFFFFFFFF)
_PHILOX_M0 = np.uint64(0xD2511F53)
_PHILOX_M1 = np.uint64(0xCD9E8D57)
_PHILOX_W0 = 0x9E3779B9
_PHILOX_W1 = 0xBB67AE85


# ----------------------------------------------------------------------------
# Philox4x32-10 (this project's stream; published algorithm, SC'11)
# ----------------------------------------------------------------------------
def philox4x32_10(ctr, key):
    """Philox4x32 with 10 rounds.  ``ctr`` is four uint32 arrays (broadcastable),
    ``key`` two Python ints.  Returns four uint32 arrays."""
    c0, c1, c2, c3 = (np.asarray(c, dtype=np.uint64) & _MASK32 for c in ctr)
    k0 = int(key[0]) & 0xFFFFFFFF
    k1 = int(key[1]) & 0xFFFFFFFF
    for _ in range(10):
        p0 = _PHILOX_M0 * c0
        p1 = _PHILOX_M1 * c2
        hi0, lo0 = p0 >> np.uint64(32), p0 & _MASK32
        hi1, lo1 = p1 >> np.uint64(32), p1 & _MASK32
        c0, c1, c2, c3 = hi1 ^ c1 ^ np.uint64(k0), lo1, hi0 ^ c3 ^ np.uint64(k1), lo0
        k0 = (k0 + _PHILOX_W0) & 0xFFFFFFFF
        k1 = (k1 + _PHILOX_W1) & 0xFFFFFFFF
    return tuple(c.astype(np.uint32) for c in (c0, c1, c2, c3))


def philox_words(seed, call_ctr, ev_offset, n, n_words):
    """The (n, n_words) uint32 words the GPU sampler draws for events
    ``ev_offset .. ev_offset+n-1`` of sampler call ``call_ctr``.

    Counter layout (one 4-word block per ``q``): ``(ev & 0xffffffff, ev >> 32,
    (call_ctr << 4 | q) & 0xffffffff, call_ctr >> 28)``; key = the 64-bit seed.
    """
    ev = np.arange(ev_offset, ev_offset + n, dtype=np.uint64)
    key = (seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF)
    out = np.empty((n, 4 * ((n_words + 3) // 4)), dtype=np.uint32)
    for q in range((n_words + 3) // 4):
        c2 = ((call_ctr << 4) | q) & 0xFFFFFFFF
        c3 = (call_ctr >> 28) & 0xFFFFFFFF
        r = philox4x32_10((ev & _MASK32, ev >> np.uint64(32), np.uint64(c2), np.uint64(c3)), key)
        for j in range(4):
            out[:, 4 * q + j] = r[j]
    return out[:, :n_words]


def words_to_u53(w_hi, w_lo):
    """53-bit uniform in [0, 1) from two 32-bit words: ((hi>>5)*2^26 + (lo>>6)) * 2^-53."""
    a = (np.asarray(w_hi, dtype=np.uint64) >> np.uint64(5)).astype(np.float64)
    b = (np.asarray(w_lo, dtype=np.uint64) >> np.uint64(6)).astype(np.float64)
    return (a * 67108864.0 + b) * (1.0 / 9007199254740992.0)


def tech_cut_affine(u01):
    """U[0,1) -> U[TECH_CUT, 1-TECH_CUT): ``u * (maxval - minval) + minval`` as two
    float64 roundings, the form ``tf.random.uniform`` applies to its raw draws
    (monte_carlo.py:264-266)."""
    maxval = np.float64(1.0 - TECH_CUT)
    minval = np.float64(TECH_CUT)
    rng = maxval - minval
    u = np.asarray(u01, dtype=np.float64)
    return (u * rng) + minval


def uniforms_f64_philox(seed, call_ctr, ev_offset, n, n_dim):
    """The (n, n_dim) float64 uniforms (post TECH_CUT affine) of the GPU's
    float64 sampler: dimension d uses words 2d (high) and 2d+1 (low)."""
    w = philox_words(seed, call_ctr, ev_offset, n, 2 * n_dim)
    u = words_to_u53(w[:, 0::2], w[:, 1::2])
    return tech_cut_affine(u)


# ----------------------------------------------------------------------------
# Importance-sampling map
# ----------------------------------------------------------------------------
def initial_grid(n_dim):
    """vflow.py:239-242: ``linspace(0, 1, 51)`` for every dimension."""
    sub = np.linspace(0, 1, BINS_MAX + 1)
    return sub.repeat(n_dim).reshape(-1, n_dim).T.copy()


def importance_sampling_digest(xn, divisions):
    """vflow.py:39-83.  ``xn`` (n_dim, n) float64, ``divisions`` (n_dim, 51).

    Returns ``ind`` (n, n_dim) int32, ``x`` (n, n_dim) float64, ``w`` (n,)."""
    ind_i = xn.astype(np.int32)                                   # :67 (trunc)
    ind_f = ind_i + 1                                             # :69
    x_ini = np.take_along_axis(divisions, ind_i, axis=1)          # :70
    x_fin = np.take_along_axis(divisions, ind_f, axis=1)          # :71
    xdelta = x_fin - x_ini                                        # :73
    aux_rand = xn - np.floor(xn)                                  # :75
    x = x_ini + xdelta * aux_rand                                 # :76
    fac = xdelta * float(BINS_MAX)                                # :78 (product over dims,
    weights = fac[0].copy()                                       #      in dimension order)
    for d in range(1, fac.shape[0]):
        weights = weights * fac[d]
    return ind_i.T.copy(), x.T.copy(), weights                    # :81-82


def vegas_map(rnds, divisions):
    """vflow.py:93-126: ``xn = 50 * (1 - rnds^T)`` then the digest."""
    xn = float(BINS_MAX) * (1.0 - np.asarray(rnds, dtype=np.float64).T)
    ind, x, w = importance_sampling_digest(xn, divisions)
    return x, w, ind


def plus_map(rnds, n_strat, n_ev, divisions):
    """vflowplus.py:46-80: events laid out hypercube by hypercube (``n_ev[h]`` each),
    ``xn = (p + u)^T * 50 / n_strat``, digest, weight divided by ``n_ev[h]``.

    Hypercube ``h`` has coordinates given by ``itertools.product(range(n_strat),
    repeat=n_dim)`` order (last dimension fastest), vflowplus.py:126-128."""
    rnds = np.asarray(rnds, dtype=np.float64)
    n_dim = rnds.shape[1]
    n_ev = np.asarray(n_ev, dtype=np.int64)
    h = np.repeat(np.arange(n_ev.size), n_ev)                          # :67
    points = np.empty((h.size, n_dim), dtype=np.float64)               # :68
    rem = h.copy()
    for d in range(n_dim - 1, -1, -1):
        points[:, d] = rem % n_strat
        rem //= n_strat
    n_evs = n_ev[h].astype(np.float64)                                 # :69
    xn = (points + rnds).T * float(BINS_MAX) / float(n_strat)          # :72
    ind, x, w = importance_sampling_digest(xn, divisions)              # :74
    return x, w / n_evs, ind, h                                        # :77


def consume_array_into_indices(input_arr, indices, result_size):
    """utils.py:17-44: per-bin sum of ``input_arr`` by ``indices`` (n,) or (n,1)."""
    idx = np.asarray(indices).reshape(-1)
    return np.bincount(idx, weights=np.asarray(input_arr, dtype=np.float64),
                       minlength=int(result_size))[: int(result_size)]


# ----------------------------------------------------------------------------
# Grid refinement (vflow.py:135-211)
# ----------------------------------------------------------------------------
def refine_grid_per_dimension(t_res_sq, subdivisions, return_flag=False):
    """Smear, damp (alpha=1.5), and rebin one dimension.  Returns the 51 new edges.

    The rebinning walks bins exactly as the reference's ``tf.while_loop``: the
    state (bin_weight, n_bin, cur, prev) carries over the 49 outer steps.  If
    rounding would push ``n_bin`` past the last bin (the reference would index
    out of range), the walk stops at bin 49 and ``flag`` is set."""
    r = np.asarray(t_res_sq, dtype=np.float64)
    sub = np.asarray(subdivisions, dtype=np.float64)
    meaner = np.full(BINS_MAX, 3.0)
    meaner[0] = meaner[-1] = 2.0                                       # :152-154
    pad = np.zeros(BINS_MAX + 2)
    pad[1:-1] = r                                                      # :156
    smeared = np.maximum((pad[1:-1] + pad[2:] + pad[:-2]) / meaner, 1e-30)  # :158-159
    sum_t = np.sum(smeared)                                            # :162
    log_t = np.log(smeared)                                            # :163
    aux_t = (1.0 - smeared / sum_t) / (np.log(sum_t) - log_t)          # :164
    wei_t = np.power(aux_t, ALPHA)                                     # :165
    ave_t = np.sum(wei_t) / BINS_MAX                                   # :166
    new_bins = [0.0]
    bin_weight = 0.0
    n_bin = -1
    cur = 0.0
    prev = 0.0
    flag = 0
    for _ in range(BINS_MAX - 1):                                      # :201-207
        while bin_weight < ave_t:
            if n_bin + 1 >= BINS_MAX:
                flag = 1
                break
            n_bin += 1
            bin_weight += wei_t[n_bin]
            prev = cur
            cur = sub[n_bin + 1]
        bin_weight -= ave_t
        delta = (cur - prev) * bin_weight / wei_t[n_bin]
        new_bins.append(cur - delta)
    new_bins.append(1.0)
    out = np.array(new_bins, dtype=np.float64)
    return (out, flag) if return_flag else out


def refine_grid(arr_res2, divisions):
    """vflow.py:349-362: refine every dimension; returns the new (n_dim, 51) grid."""
    return np.stack([refine_grid_per_dimension(arr_res2[j], divisions[j])
                     for j in range(divisions.shape[0])])


# ----------------------------------------------------------------------------
# Integrands (config workloads)
# ----------------------------------------------------------------------------
def integrand_symgauss(x, a=0.1):
    """Normalised symmetric Gaussian prod_d exp(-(x-1/2)^2/a^2)/(a sqrt(pi))
    (the reference tests' integrand, simgauss_tf.py:22-32, without the
    constant terms that cancel)."""
    n_dim = x.shape[-1]
    pref = (1.0 / a / np.sqrt(np.pi)) ** n_dim
    coef = np.zeros(x.shape[0])
    for d in range(n_dim):
        t = (x[:, d] - 0.5) / a
        coef = coef + t * t
    return pref * np.exp(-coef)


def symgauss_exact(n_dim, a=0.1):
    return math.erf(0.5 / a) ** n_dim


def integrand_gauss_mu(x, mu, a):
    """Unnormalised Gaussian prod_d exp(-(x_d-mu_d)^2/a_d^2) (batched workload)."""
    coef = np.zeros(x.shape[0])
    for d in range(x.shape[1]):
        t = (x[:, d] - mu[d]) / a[d]
        coef = coef + t * t
    return np.exp(-coef)


def gauss_mu_exact(mu, a):
    out = 1.0
    for m, s in zip(mu, a):
        out *= s * math.sqrt(math.pi) / 2.0 * (math.erf((1.0 - m) / s) + math.erf(m / s))
    return out


def integrand_breit_wigner(x, mass=91.19, width=2.50, coeffs=None):
    """Breit-Wigner in s = 2500 + 20000 x_1 (Jacobian 20000 included) times
    prod_{d>=2} (1 + c_d x_d)."""
    s = 2500.0 + 20000.0 * x[:, 0]
    m2 = mass * mass
    ds = s - m2
    f = 20000.0 / (ds * ds + m2 * width * width)
    for d in range(1, x.shape[1]):
        f = f * (1.0 + coeffs[d - 1] * x[:, d])
    return f


def breit_wigner_exact(n_dim, mass=91.19, width=2.50, coeffs=None):
    mg = mass * width
    m2 = mass * mass
    val = (math.atan((22500.0 - m2) / mg) - math.atan((2500.0 - m2) / mg)) / mg
    for d in range(1, n_dim):
        val *= 1.0 + coeffs[d - 1] / 2.0
    return val


def integrand_prod(x):
    """test_misc.py:24-26 ``_simple_integrand``: prod_d x_d."""
    out = x[:, 0].copy()
    for d in range(1, x.shape[1]):
        out = out * x[:, d]
    return out


def integrand_sum(x):
    """examples/cuda: sum_d x_d."""
    out = x[:, 0].copy()
    for d in range(1, x.shape[1]):
        out = out + x[:, d]
    return out


INTEGRANDS = {
    "symgauss": integrand_symgauss,
    "gauss_mu": integrand_gauss_mu,
    "breit_wigner": integrand_breit_wigner,
    "prod": integrand_prod,
    "sum": integrand_sum,
}


# ----------------------------------------------------------------------------
# Drivers
# ----------------------------------------------------------------------------
def chunk_sizes(n_events, events_per_run):
    """monte_carlo.py:437-452: the per-step event counts of one iteration."""
    out = []
    left = n_events
    while left > 0:
        out.append(min(left, events_per_run))
        left -= events_per_run
    return out


def weighted_average(history):
    """monte_carlo.py:712-732: 1/sigma^2-weighted mean and its sigma."""
    aux_res = 0.0
    weight_sum = 0.0
    for res, sigma in history:
        wgt_tmp = 1.0 / pow(sigma, 2)
        aux_res += res * wgt_tmp
        weight_sum += wgt_tmp
    return aux_res / weight_sum, float(np.sqrt(1.0 / weight_sum))


class _OracleBase:
    def __init__(self, n_dim, n_events, events_limit=MAX_EVENTS_LIMIT, xmin=None, xmax=None):
        self.n_dim = n_dim
        self.n_events = int(n_events)
        self.events_limit = int(events_limit)
        self.history = []
        if xmin is not None or xmax is not None:                       # monte_carlo.py:159-171
            if xmin is None or xmax is None:
                raise ValueError("Both xmin and xmax must be provided")
            if not (len(xmin) == len(xmax) == n_dim):
                raise ValueError("The integration limits must be given for all dimensions")
            self.xmin = np.asarray(xmin, dtype=np.float64)
            self.xdelta = np.asarray(xmax, dtype=np.float64) - self.xmin
            if np.any(self.xdelta < 0.0):
                raise ValueError("xmin > xmax")
            jac = self.xdelta[0]
            for d in range(1, n_dim):
                jac = jac * self.xdelta[d]
            self.xdeltajac = jac
        else:
            self.xmin = self.xdelta = self.xdeltajac = None

    @property
    def events_per_run(self):
        return min(self.events_limit, self.n_events)

    @property
    def xjac(self):
        """monte_carlo.py:225-227."""
        return 1.0 / self.n_events

    def _finish_weights(self, x, w):
        """monte_carlo.py:270-274."""
        w = w * self.xjac
        if self.xdelta is not None:
            x = self.xmin + x * self.xdelta
            w = w * self.xdeltajac
        return x, w

    def run_integration(self, n_iter, uniform_source, integrand):
        for _ in range(n_iter):
            self.history.append(self.iteration(uniform_source, integrand))
        return weighted_average(self.history)


class OracleVegas(_OracleBase):
    """VegasFlow (vflow.py:215-446) driven by an explicit uniform source.

    ``uniform_source(n, n_dim)`` returns the post-affine uniforms of the next
    ``n`` events (called once per event chunk, in order)."""

    def __init__(self, n_dim, n_events, train=True, **kw):
        super().__init__(n_dim, n_events, **kw)
        self.train = train
        self.divisions = initial_grid(n_dim)
        self.last = None

    def sample(self, rnds):
        x, w, ind = vegas_map(rnds, self.divisions)
        x, w = self._finish_weights(x, w)
        return x, w, ind

    def run_event(self, rnds, integrand):
        """vflow.py:389-430 for one chunk: returns res, res2, arr_res2 (+ taps)."""
        x, w, ind = self.sample(rnds)
        f = integrand(x)
        tmp = w * f
        tmp2 = tmp * tmp
        res = np.sum(tmp)
        res2 = np.sum(tmp2)
        arr = np.stack([consume_array_into_indices(tmp2, ind[:, j], BINS_MAX)
                        for j in range(self.n_dim)]) if self.train else None
        return res, res2, arr, dict(x=x, w=w, ind=ind, f=f)

    def iteration(self, uniform_source, integrand):
        """vflow.py:432-442 with monte_carlo.py:420-480 chunking."""
        res = res2 = 0.0
        arr = np.zeros((self.n_dim, BINS_MAX))
        taps = []
        for nc in chunk_sizes(self.n_events, self.events_per_run):
            r, r2, a, t = self.run_event(uniform_source(nc, self.n_dim), integrand)
            res += r
            res2 += r2
            if a is not None:
                arr += a
            taps.append(t)
        n = self.n_events
        err_tmp2 = (n * res2 - res * res) / (n - 1.0)
        sigma = float(np.sqrt(max(err_tmp2, 0.0)))
        self.last = dict(res=res, res2=res2, arr_res2=arr, taps=taps,
                         grid_before=self.divisions.copy())
        if self.train:
            self.divisions = refine_grid(arr, self.divisions)
        return float(res), sigma


class OraclePlain(_OracleBase):
    """PlainFlow (plain.py:11-43)."""

    def iteration(self, uniform_source, integrand):
        res = raw_res2 = 0.0
        for nc in chunk_sizes(self.n_events, self.events_per_run):
            x, w = self._finish_weights(uniform_source(nc, self.n_dim), np.float64(1.0))
            tmp = integrand(x) * w
            res += np.sum(tmp)
            raw_res2 += np.sum(tmp * tmp)
        res2 = raw_res2 * self.n_events
        err_tmp2 = (res2 - res * res) / (self.n_events - 1.0)
        return float(res), float(np.sqrt(max(err_tmp2, 0.0)))


def plus_stratification(n_dim, n_events, adaptive):
    """vflowplus.py:103-139: (adaptive, n_strat, n_hypercubes, min_neval, n_events).

    The powers are taken in float32, as TensorFlow does for Python-float operands."""
    if n_dim > 13 and adaptive:
        adaptive = False
    if adaptive:
        neval_eff = int(n_events / 2)
    else:
        neval_eff = n_events
    n_strat = np.floor(np.power(np.float32(neval_eff / 2), np.float32(1 / n_dim)))
    if np.power(np.float32(n_strat), np.float32(n_dim)) > MAX_NEVAL_HCUBE:
        n_strat = np.floor(np.power(np.float32(1e4), np.float32(1 / n_dim)))
    n_strat = int(n_strat)
    n_hcubes = n_strat ** n_dim
    min_neval = max(int(neval_eff // n_hcubes), 2)
    return adaptive, n_strat, n_hcubes, min_neval, min_neval * n_hcubes


def redistribute_samples(arr_var, min_neval, init_calls):
    """vflowplus.py:153-163.  ``tf.maximum(min, nan)`` returns ``min`` (the NaN of
    a rounding-negative variance loses), hence ``fmax``."""
    with np.errstate(invalid="ignore"):
        damped = np.power(arr_var, BETA / 2)
    new = np.fmax(float(min_neval), damped * float(init_calls) / 2 / np.sum(damped))
    n_ev = new.astype(np.int32)
    return n_ev, int(np.sum(n_ev))


class OraclePlus(OracleVegas):
    """VegasFlowPlus (vflowplus.py:83-247)."""

    def __init__(self, n_dim, n_events, train=True, adaptive=False, **kw):
        kw.pop("events_limit", None)
        super().__init__(n_dim, n_events, train=train, events_limit=n_events, **kw)
        self.init_calls = int(n_events)
        (self.adaptive, self.n_strat, self.n_hcubes, self.min_neval,
         n_tot) = plus_stratification(n_dim, n_events, adaptive)
        self.n_ev = np.full(self.n_hcubes, self.min_neval, dtype=np.int32)
        self.n_events = n_tot

    @property
    def xjac(self):
        return 1.0 / self.n_hcubes                                      # :139, :144-146

    def iteration(self, uniform_source, integrand):
        rnds = uniform_source(self.n_events, self.n_dim)
        x, w, ind, seg = plus_map(rnds, self.n_strat, self.n_ev, self.divisions)
        x, w = self._finish_weights(x, w)
        f = integrand(x)
        tmp = w * f                                                     # :209
        tmp2 = tmp * tmp
        ress = np.bincount(seg, weights=tmp, minlength=self.n_hcubes)   # :213
        ress2 = np.bincount(seg, weights=tmp2, minlength=self.n_hcubes)
        arr_var = ress2 * self.n_ev.astype(np.float64) - ress * ress   # :216-217
        arr = np.stack([consume_array_into_indices(tmp2, ind[:, j], BINS_MAX)
                        for j in range(self.n_dim)])
        sigmas2 = np.maximum(arr_var, 0.0)                              # :230-233
        res = np.sum(ress)
        sigma2 = np.sum(sigmas2 / (self.n_ev.astype(np.float64) - 1.0))
        sigma = float(np.sqrt(sigma2))
        self.last = dict(res=res, ress=ress, ress2=ress2, arr_var=arr_var, arr_res2=arr,
                         n_ev=self.n_ev.copy(), grid_before=self.divisions.copy(),
                         taps=[dict(x=x, w=w, ind=ind, f=f)])
        if self.adaptive:                                               # :236-237
            self.n_ev, self.n_events = redistribute_samples(arr_var, self.min_neval,
                                                            self.init_calls)
        if self.train:                                                  # :239-240
            self.divisions = refine_grid(arr, self.divisions)
        return float(res), sigma


# ----------------------------------------------------------------------------
# float32 fused-form map (the GPU's fp32 sampler on Philox words)
# ----------------------------------------------------------------------------
def _f32_frac_from_lo(lo):
    """float32 in [0, 1): the top 23 bits of a 32-bit word, via the [1, 2) bit pattern."""
    bits = (np.asarray(lo, dtype=np.uint32) >> np.uint32(9)) | np.uint32(0x3F800000)
    return bits.view(np.float32) - np.float32(1.0)


def fma_f32(a, b, c):
    """float32(a * b + c) with one rounding (a, b, c float32 arrays): the product
    is exact in float64 (24 + 24 bits), the sum's float64 rounding error is
    recovered by TwoSum and folded in as a round-to-odd of the float64 sum, after
    which the conversion to float32 rounds as a single fused operation would."""
    p = a.astype(np.float64) * b.astype(np.float64)
    c64 = c.astype(np.float64)
    s = p + c64
    bb = s - p
    err = (p - (s - bb)) + (c64 - bb)
    even = (s.view(np.uint64) & np.uint64(1)) == 0
    fix = (err != 0.0) & even
    s = np.where(fix, np.nextafter(s, s + err), s)
    return s.astype(np.float32)


def f32_weight_prescale(c1):
    """Exponent k of the fp32 samplers' power-of-two weight prescale 2^k for the
    float64 bin widths ``c1`` (any shape, all D x 50 cells): the sum of their
    binary exponents, each clamped to float32's normal range [-126, 127] (a zero
    width counts as -126), divided by 50 in float32, rounded to the nearest
    integer (ties to even), negated and clamped to [-100, 100]."""
    bits = np.asarray(c1, dtype=np.float64).view(np.uint64)
    e = ((bits >> np.uint64(52)) & np.uint64(0x7FF)).astype(np.int64) - 1023
    expsum = int(np.clip(e, -126, 127).sum())
    k = -int(np.rint(np.float32(expsum) / np.float32(BINS_MAX)))
    return max(-100, min(100, k))


def vegas_map_f32_words(words, divisions, xjac, xmin=None, xdelta=None):
    """fp32 form of the importance map on one 32-bit Philox word per dimension
    (the fused sampler's and the map kernel's draw, no integration limits).

    With u = (word + 1/2) / 2^32: ``p = 50 * word + 25`` (exact, 64-bit) is
    50 u 2^32, so ``j = p >> 32`` is floor(50 u) and ``ind = 49 - j`` the
    reference's ``int32(50 (1 - u))`` (vflow.py:117, :67; exact in float64 for
    such u); ``m = 1 + (top 23 bits of p mod 2^32) / 2^23`` is 1 + frac(50 u).
    The table is reversed: with c0 = lo - delta and c1 = delta (float64), the
    cell of bin b holds ``C0 = f32(fma64(3, c1, c0))`` and ``C1 = f32(-c1)``, so
    that ``x = fl32(C1 m + C0)`` (one fused multiply-add) is
    lo + delta (1 - frac(50 u)), the reference's lo + delta frac.  The weight is
    2^k C1_0 C1_1 ... C1_{D-1} in float32 left to right (k from
    ``f32_weight_prescale``) times the float32 constant
    ``(-1)^D xjac 50^D 2^-k`` (its float64 product rounded once).  With
    integration limits (monte_carlo.py:169-176, 270-273) the cell's affine
    coefficients are ``c0 = fma64(lo - delta, xdelta, xmin)`` and
    ``c1 = delta xdelta`` before the table is formed, so x is in the limits'
    box and the weight carries the volume.
    Returns (ind int32, x float32, w float32)."""
    from fractions import Fraction
    words = np.asarray(words, dtype=np.uint32)
    n, n_dim = words.shape
    p = words.astype(np.uint64) * np.uint64(50) + np.uint64(25)
    j = (p >> np.uint64(32)).astype(np.int32)
    ind = (BINS_MAX - 1 - j).astype(np.int32)
    mbits = ((p & _MASK32) >> np.uint64(9)).astype(np.uint32) | np.uint32(0x3F800000)
    m = mbits.view(np.float32)
    g = np.asarray(divisions, dtype=np.float64)
    lo = g[:, :-1]
    c1 = g[:, 1:] - lo
    c0 = lo - c1
    if xmin is not None:
        xmin = np.asarray(xmin, dtype=np.float64)
        xdelta = np.asarray(xdelta, dtype=np.float64)
        c0 = np.array([[float(Fraction(float(a)) * Fraction(float(xdelta[d])) + Fraction(float(xmin[d])))
                        for a in c0[d]] for d in range(n_dim)])
        c1 = c1 * xdelta[:, None]
    # fma64(3, c1, c0) rounded to float64 once (exact rational sum, nearest-even)
    big = np.array([[float(Fraction(3) * Fraction(float(b)) + Fraction(float(a))) for a, b in zip(ra, rb)]
                    for ra, rb in zip(c0, c1)])
    C0 = big.astype(np.float32)
    C1 = (-c1).astype(np.float32)
    c0e = np.take_along_axis(C0, ind.T, axis=1).T
    c1e = np.take_along_axis(C1, ind.T, axis=1).T
    x = fma_f32(c1e, m, c0e)
    k = f32_weight_prescale(c1)
    wf = (np.float32(2.0 ** k) * c1e[:, 0]).astype(np.float32)
    for d in range(1, n_dim):
        wf = (wf * c1e[:, d]).astype(np.float32)
    ws = -float(xjac) if n_dim & 1 else float(xjac)
    for _ in range(n_dim):
        ws *= 50.0
    w = (wf * np.float32(ws * 2.0 ** -k)).astype(np.float32)
    return ind, x, w


def uniforms_of_words(words):
    """The float64 uniforms ``u = (word + 1/2) / 2^32`` that the fp32 samplers'
    integer maps stand for (exact in float64)."""
    return (np.asarray(words, dtype=np.float64) + 0.5) / 4294967296.0


def plus_bins_from_words(words, points, n_strat):
    """The fp32 VEGAS+ sampler's stratified bin per dimension, in exact integer
    arithmetic: ``Q = 50 (p 2^32 + word) + 25`` is ``50 (p + u) 2^32`` for
    u = (word + 1/2) / 2^32, and ``bin = (Q >> 32) div n_strat`` is
    ``floor((p + u) 50 / n_strat)`` (vflowplus.py:72)."""
    w = np.asarray(words, dtype=np.uint64)
    p = np.asarray(points, dtype=np.uint64)
    Q = ((p << np.uint64(32)) | w) * np.uint64(50) + np.uint64(25)
    return ((Q >> np.uint64(32)) // np.uint64(int(n_strat))).astype(np.int32)


def plus_map_f32_words(words, points, n_strat, divisions):
    """The fp32 VEGAS+ sampler's points (no integration limits): with
    Q = 50 (p 2^32 + word) + 25, A = Q >> 32, R = Q mod 2^32, bin i = A div
    n_strat and r = A mod n_strat (``plus_bins_from_words``), the fraction plus 1
    is ``m = fl32(fl32(R 2^-32 + r) / n_strat + 1)`` with the division by a
    float32 reciprocal and both steps fused multiply-adds, capped below 2, and
    ``x = fl32(c1 m + c0)`` through the per-bin table ``c0 = f32(lo - delta)``,
    ``c1 = f32(delta)`` (each rounded once from float64).  Returns x float32."""
    w = np.asarray(words, dtype=np.uint64)
    p = np.asarray(points, dtype=np.uint64)
    ns = int(n_strat)
    Q = ((p << np.uint64(32)) | w) * np.uint64(50) + np.uint64(25)
    A = Q >> np.uint64(32)
    R = (Q & _MASK32).astype(np.uint32)
    i = (A // np.uint64(ns)).astype(np.int64)
    r = (A - (A // np.uint64(ns)) * np.uint64(ns)).astype(np.float32)
    inv_ns = np.float32(1.0) / np.float32(ns)
    t = fma_f32(R.astype(np.float32), np.full(R.shape, np.float32(2.0 ** -32)), r)
    m = fma_f32(t, np.full(t.shape, inv_ns), np.ones(t.shape, dtype=np.float32))
    m = np.minimum(m, np.float32(1.99999988))
    g = np.asarray(divisions, dtype=np.float64)
    lo = g[:, :-1]
    dl = g[:, 1:] - lo
    c0 = (lo - dl).astype(np.float32)
    c1 = dl.astype(np.float32)
    c0e = np.take_along_axis(c0, i.T, axis=1).T
    c1e = np.take_along_axis(c1, i.T, axis=1).T
    return fma_f32(c1e, m, c0e)


def plain_map_f32_words(words):
    """fp32 plain-MC uniform: top 23 bits as [0,1) plus 2^-24."""
    return _f32_frac_from_lo(words) + np.float32(2.0 ** -24)


# ----------------------------------------------------------------------------
# Threaded CPU run (the CPU baseline): one VegasFlow iteration split in chunks
# ----------------------------------------------------------------------------
def threaded_vegas_iteration(divisions, n_events, integrand, seed, n_threads, chunk=MAX_EVENTS_LIMIT):
    """One float64 VegasFlow iteration on ``n_threads`` host threads, each chunk
    drawing NumPy uniforms (PCG64) through the TECH_CUT affine.  Returns
    (res, sigma, arr_res2).  NumPy releases the GIL inside the array kernels."""
    n_dim = divisions.shape[0]
    sizes = chunk_sizes(n_events, chunk)
    xjac = 1.0 / n_events

    def work(i):
        rng = np.random.default_rng([seed, i])
        rnds = tech_cut_affine(rng.random((sizes[i], n_dim)))
        x, w, ind = vegas_map(rnds, divisions)
        w = w * xjac
        tmp = w * integrand(x)
        tmp2 = tmp * tmp
        arr = np.stack([np.bincount(ind[:, j], weights=tmp2, minlength=BINS_MAX)
                        for j in range(n_dim)])
        return np.sum(tmp), np.sum(tmp2), arr

    with ThreadPoolExecutor(max_workers=n_threads) as ex:
        parts = list(ex.map(work, range(len(sizes))))
    res = sum(p[0] for p in parts)
    res2 = sum(p[1] for p in parts)
    arr = sum(p[2] for p in parts)
    err = (n_events * res2 - res * res) / (n_events - 1.0)
    return res, float(np.sqrt(max(err, 0.0))), arr


def hypercube_points(n_hcubes, n_strat, n_dim):
    """vflowplus.py:126-128 ordering, for tests."""
    return np.array(list(product(range(n_strat), repeat=n_dim)), dtype=np.int32)[:n_hcubes]
