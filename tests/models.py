"""Seeded model Hamiltonians (re-exported from the package for the tests)."""
from chemps2_gb300.models import NIRREPS, Model, bcs, hubbard, synthetic_ab_initio  # noqa: F401
