"""Seeded synthetic datasets for the tests, plus their oracle models (the
oracle is constructed here, in the tests, never by the package)."""
import oracle
from stan_gb300 import workloads
from stan_gb300.workloads import Dataset


def _oracle_model(self, compensated=True):
    return oracle.OracleModel(self.kind, self.X, self.y, group=self.group, J=self.J,
                              hp=list(self.hp), intercept=self.intercept, compensated=compensated)


Dataset.oracle_model = _oracle_model


def make_dataset(kind, small=False, seed=1):
    return workloads.make_dataset(kind, small=small, seed=seed)


def logistic_laplace_draws(ds, n, seed=0):
    """n draws from the Laplace approximation of a logistic GLM's posterior
    (Newton mode of the log density, covariance the inverse negative
    Hessian): posterior-region points without running a sampler.  With
    N = 1e5 rows the posterior is close to this normal."""
    import numpy as np
    X = np.hstack([np.ones((ds.N, 1)), ds.X]) if ds.intercept else ds.X
    s2 = ds.hp[0] ** 2
    th = np.zeros(X.shape[1])
    for _ in range(50):
        p = 1.0 / (1.0 + np.exp(-(X @ th)))
        g = X.T @ (ds.y - p) - th / s2
        H = (X * (p * (1 - p))[:, None]).T @ X + np.eye(X.shape[1]) / s2
        step = np.linalg.solve(H, g)
        th = th + step
        if np.max(np.abs(step)) < 1e-12:
            break
    L = np.linalg.cholesky(np.linalg.inv(H))
    z = np.random.default_rng(seed).normal(size=(X.shape[1], n))
    return th + (L @ z).T
