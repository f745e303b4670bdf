"""Seeded synthetic datasets for the four log densities and the workloads they
are benchmarked on (no public dataset is named for this path, so inputs are
generated with the stated shapes and distributions).

  logistic_1k    : N=1000,   K=25,  X ~ N(0,1) FP64, alpha, beta ~ N(0,1)
  logistic_100k  : N=100000, K=100, X ~ N(0,1) columns standardised, stored FP32
  hier_normal    : J=2000 groups, n_j = 1 + Poisson(20), K=10, mu=1, tau=0.5,
                   sigma=1, beta, z ~ N(0,1); rows sorted by group
  poisson_262k   : N=262144, K=512, X ~ N(0, 1/K) stored BF16, beta ~ N(0, 0.5)
  hier_logistic  : serving fits, N log-uniform [200, 5e4], K in {8..128}, J = N/50,
                   y drawn at prior draws
"""
import dataclasses
import math

import numpy as np

LOGISTIC, POISSON, HIER_NORMAL, HIER_LOGISTIC = 1, 2, 3, 4
KIND_CODES = {"logistic": LOGISTIC, "poisson": POISSON, "hier_normal": HIER_NORMAL,
              "hier_logistic": HIER_LOGISTIC}


def round_to_bf16(x):
    """Round float64 values to the nearest bfloat16 (ties to even), returned as float64."""
    f = np.ascontiguousarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    lsb = (u >> np.uint64(16)) & np.uint64(1)
    u = (u + np.uint64(0x7FFF) + lsb) & np.uint64(0xFFFF0000)
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


@dataclasses.dataclass
class Dataset:
    name: str
    kind: int
    X: np.ndarray            # (N, K) float64; values exactly representable in x_dtype
    y: np.ndarray            # (N,) float64
    x_dtype: str = "f64"     # storage type on the device: f64 | f32 | bf16
    group: np.ndarray = None  # (N,) int32 group of each row (sorted), hierarchical only
    J: int = 0
    hp: tuple = ()
    intercept: bool = True
    truth: np.ndarray = None

    @property
    def N(self):
        return self.X.shape[0]

    @property
    def K(self):
        return self.X.shape[1]

    @property
    def D(self):
        if self.kind in (LOGISTIC, POISSON):
            return self.K + (1 if self.intercept else 0)
        if self.kind == HIER_NORMAL:
            return 3 + self.J + self.K
        return 2 + self.J + self.K

    def param_names(self):
        K, J = self.K, self.J
        if self.kind in (LOGISTIC, POISSON):
            return (["alpha"] if self.intercept else []) + [f"beta.{k + 1}" for k in range(K)]
        if self.kind == HIER_NORMAL:
            return ["mu", "tau", "sigma"] + [f"z.{j + 1}" for j in range(J)] + [f"beta.{k + 1}" for k in range(K)]
        return ["alpha", "tau"] + [f"z.{j + 1}" for j in range(J)] + [f"beta.{k + 1}" for k in range(K)]


def _groups(rng, J, mean_size):
    sizes = 1 + rng.poisson(mean_size - 1, size=J)
    return np.repeat(np.arange(J, dtype=np.int32), sizes)


def logistic(N=1000, K=25, seed=1, x_dtype="f64", standardise=False, name=None):
    rng = np.random.default_rng(seed)
    X = rng.normal(size=(N, K))
    if standardise:
        X = (X - X.mean(0)) / X.std(0)
    if x_dtype == "f32":
        X = X.astype(np.float32).astype(np.float64)
    elif x_dtype == "bf16":
        X = round_to_bf16(X)
    alpha = rng.normal()
    beta = rng.normal(size=K)
    eta = alpha + X @ beta
    y = (rng.random(N) < 1 / (1 + np.exp(-eta))).astype(np.float64)
    return Dataset(name or f"logistic_N{N}_K{K}", LOGISTIC, X, y, x_dtype, hp=(2.5,),
                   truth=np.concatenate([[alpha], beta]))


def poisson(N=262144, K=512, seed=1, x_dtype="bf16", name=None):
    rng = np.random.default_rng(seed)
    X = rng.normal(scale=1 / math.sqrt(K), size=(N, K))
    if x_dtype == "bf16":
        X = round_to_bf16(X)
    elif x_dtype == "f32":
        X = X.astype(np.float32).astype(np.float64)
    beta = rng.normal(scale=0.5, size=K)
    y = rng.poisson(np.exp(X @ beta)).astype(np.float64)
    return Dataset(name or f"poisson_N{N}_K{K}", POISSON, X, y, x_dtype, hp=(1.0,),
                   intercept=False, truth=beta)


def hier_normal(J=2000, K=10, mean_size=21, seed=1, x_dtype="f64", name=None):
    rng = np.random.default_rng(seed)
    g = _groups(rng, J, mean_size)
    N = g.size
    X = rng.normal(size=(N, K))
    if x_dtype == "f32":
        X = X.astype(np.float32).astype(np.float64)
    mu, tau, sigma = 1.0, 0.5, 1.0
    beta = rng.normal(size=K)
    z = rng.normal(size=J)
    y = mu + tau * z[g] + X @ beta + sigma * rng.normal(size=N)
    truth = np.concatenate([[mu, math.log(tau), math.log(sigma)], z, beta])
    return Dataset(name or f"hier_normal_J{J}_K{K}", HIER_NORMAL, X, y, x_dtype, group=g, J=J,
                   hp=(5.0, 1.0, 1.0, 1.0), truth=truth)


def hier_logistic(N=2000, K=8, seed=1, x_dtype="f32", name=None):
    rng = np.random.default_rng(seed)
    J = max(1, N // 50)
    sizes = np.full(J, N // J)
    sizes[: N - sizes.sum()] += 1
    g = np.repeat(np.arange(J, dtype=np.int32), sizes)
    X = rng.normal(size=(N, K))
    if x_dtype == "f32":
        X = X.astype(np.float32).astype(np.float64)
    alpha = rng.normal(scale=2.5)
    tau = abs(rng.normal())
    z = rng.normal(size=J)
    beta = rng.normal(scale=2.5, size=K) / math.sqrt(K)
    eta = alpha + tau * z[g] + X @ beta
    y = (rng.random(N) < 1 / (1 + np.exp(-eta))).astype(np.float64)
    truth = np.concatenate([[alpha, math.log(tau)], z, beta])
    return Dataset(name or f"hier_logistic_N{N}_K{K}", HIER_LOGISTIC, X, y, x_dtype, group=g, J=J,
                   hp=(2.5, 1.0, 2.5), truth=truth)


def hier_logistic_prior(N=2000, K=8, seed=1, name=None):
    """Hierarchical logistic data simulated at a draw from the model's own
    prior (alpha ~ N(0, 2.5), tau ~ half-N(0, 1), z ~ N(0, 1), beta ~ N(0, 2.5)),
    J = N / 50 groups, X ~ N(0, 1) stored FP32: the serving stream's fits."""
    rng = np.random.default_rng(seed)
    J = max(1, N // 50)
    sizes = np.full(J, N // J)
    sizes[: N - sizes.sum()] += 1
    g = np.repeat(np.arange(J, dtype=np.int32), sizes)
    X = rng.normal(size=(N, K)).astype(np.float32).astype(np.float64)
    alpha = rng.normal(scale=2.5)
    tau = abs(rng.normal())
    z = rng.normal(size=J)
    beta = rng.normal(scale=2.5, size=K)
    eta = alpha + tau * z[g] + X @ beta
    y = (rng.random(N) < 1 / (1 + np.exp(-eta))).astype(np.float64)
    truth = np.concatenate([[alpha, math.log(tau)], z, beta])
    return Dataset(name or f"hier_logistic_prior_N{N}_K{K}", HIER_LOGISTIC, X, y, "f32", group=g,
                   J=J, hp=(2.5, 1.0, 2.5), truth=truth)


def serving_stream(n, seed=0):
    """n serving fits: N log-uniform in [200, 50000], K uniform in {8, 16, 32,
    64, 128}, data at prior draws (hier_logistic_prior)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        N = int(round(math.exp(rng.uniform(math.log(200), math.log(50000)))))
        K = int(rng.choice([8, 16, 32, 64, 128]))
        out.append(hier_logistic_prior(N, K, seed=1000 + 7919 * seed + i))
    return out


def make_dataset(kind, small=False, seed=1):
    """The workload datasets; small=True gives a same-shaped reduced case."""
    if kind == "logistic":
        return logistic(200, 5, seed) if small else logistic(1000, 25, seed)
    if kind == "logistic_100k":
        return logistic(2000, 20, seed, "f32", True) if small else logistic(100000, 100, seed, "f32", True)
    if kind == "poisson":
        return poisson(500, 8, seed) if small else poisson(262144, 512, seed)
    if kind == "hier_normal":
        return hier_normal(20, 3, 6, seed) if small else hier_normal(2000, 10, 21, seed)
    if kind == "hier_logistic":
        return hier_logistic(300, 4, seed) if small else hier_logistic(20000, 32, seed)
    raise ValueError(kind)
