from .base import BaseFilter
from .spacial import SpacialFilter

__all__ = ["BaseFilter", "SpacialFilter"]
