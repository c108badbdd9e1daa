"""GB300-native Kohn-Sham exchange-correlation build (Chinium's src/Grid +
src/ExchangeCorrelation path) behind a C ABI; see include/chinium_xc.h."""
from ._lib import XCError, lib, PRECISION_FP64, PRECISION_MIXED
from .xc import Basis, BatchGrid, ExchangeCorrelation, Grid

__all__ = ["Basis", "Grid", "BatchGrid", "ExchangeCorrelation", "XCError", "lib", "PRECISION_FP64", "PRECISION_MIXED"]
