from skelfmm_gb300.tree import findin_sorted  # noqa: F401
