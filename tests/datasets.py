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
