from skelfmm_gb300.tree import get_point_dist, get_sphere_surface  # noqa: F401
