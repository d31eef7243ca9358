"""Stand-in for the external ``simpletree`` package, used only to run the
reference implementation when generating golden fixtures.  It re-exports the
framework's own tree (``skelfmm_gb300.tree``) under the names the reference
imports, so the fixtures and the framework share one tree definition."""
from skelfmm_gb300.tree import (  # noqa: F401
    BalancedTree,
    get_cube_surface,
    get_point_dist,
    get_sphere_surface,
)
from . import morton, morton_tree, built_in_points  # noqa: F401
