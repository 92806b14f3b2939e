"""GB300-native Liouville-space propagation (placeholder during bring-up)."""
from .constants import CM_FS, CM_FS_LINEAR, CM_K, GAUSSIAN_SD_FWHM  # noqa: F401
