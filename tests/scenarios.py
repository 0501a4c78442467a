"""Scenario builders shared by the tests (re-exported from the package's
scene module)."""
from dcgrid_gb300.scenes import (cloud, cloud256, differentiable, emission_field, heightmap, plume,  # noqa: F401
                                 plume_batch, ref_default, sphere_obstacle)
