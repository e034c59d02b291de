"""`cmtj.utils.linear` (cmtj/utils/linear.py): FieldScan."""
from ..procedures import FieldScan  # noqa: F401

__all__ = ["FieldScan"]
