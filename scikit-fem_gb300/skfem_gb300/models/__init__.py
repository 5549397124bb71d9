"""Ready-made forms (skfem/models)."""
from . import elasticity, poisson  # noqa: F401
