"""Ridge extraction on the FTLE field (drop-in for numbacs.extraction, ridge part)."""
from .ordered import ftle_ordered_ridges  # noqa: F401
from .ridges import ftle_ridge_pts, ftle_ridges, _ftle_ridges  # noqa: F401
