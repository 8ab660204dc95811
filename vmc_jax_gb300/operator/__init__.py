"""Operators (mirror of jVMC.operator)."""

from .base import Operator
from .branch_free import (BranchFreeOperator, Id, LocalOp, OpStr, Sm, Sp, Sx, Sy, Sz, annihilation, creation,
                          number, scal_opstr)

__all__ = ["Operator", "BranchFreeOperator", "Id", "LocalOp", "OpStr", "Sx", "Sy", "Sz", "Sp", "Sm",
           "number", "creation", "annihilation", "scal_opstr"]
