"""GB300-native GooFit fit path.

The GooFit host API (Observable, Variable, UnbinnedDataSet, ExpPdf,
GaussianPdf, PolynomialPdf, AddPdf, ProdPdf, ConvolutionPdf, FitManager)
over libgfengine.so: per-tree generated sm_103a kernels behind a C ABI
(include/gfengine.h).
"""
from .api import (AddPdf, CombinePdf, ConvolutionPdf, DataSet, EvalFunc, EventNumber, ExpPdf, FitManager,
                  FitManagerMinuit2, GaussianPdf, GeneralError, GooPdf, Observable, OutOfRange, PdfBase,
                  PolynomialPdf, ProdPdf, UnbinnedDataSet, Variable, get_precision, set_precision)
from .engine import Engine, FitResult, Minimizer

__all__ = [
    "AddPdf", "CombinePdf", "ConvolutionPdf", "DataSet", "EvalFunc", "EventNumber", "ExpPdf", "FitManager",
    "FitManagerMinuit2", "GaussianPdf", "GeneralError", "GooPdf", "Observable", "OutOfRange", "PdfBase",
    "PolynomialPdf", "ProdPdf", "UnbinnedDataSet", "Variable", "Engine", "FitResult", "Minimizer",
    "get_precision", "set_precision",
]
