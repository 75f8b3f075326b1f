"""Ridge extraction on the FTLE field (drop-in for numbacs.extraction, ridge part)."""
from .ridges import ftle_ridge_pts, ftle_ridges, _ftle_ridges  # noqa: F401
