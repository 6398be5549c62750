from .base import BaseFilter, DesignOps
from .helmholtz_filter_nodal import HelmholtzFilterNodal
from .spacial import SpacialFilter

__all__ = ["BaseFilter", "DesignOps", "SpacialFilter", "HelmholtzFilterNodal"]
