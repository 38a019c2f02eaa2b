"""GB300-native GooFit fit path.

The GooFit host API (Observable, Variable, UnbinnedDataSet, ExpPdf,
GaussianPdf, PolynomialPdf, AddPdf, ProdPdf, ConvolutionPdf, Amp3Body with RBW/NonRes
resonances, FitManager)
over libgfengine.so: per-tree generated sm_103a kernels behind a C ABI
(include/gfengine.h).
"""
from .api import (FF, PAIR_12, PAIR_13, PAIR_23, RBW, SF_4Body, AddPdf, Amp3Body, Amp4Body, Amplitude, AmpComponent,
                  BinnedChisqFit, BinnedDataSet, BinnedErrorFit, BinnedNllFit, FitControl, UnbinnedNllFit,
                  CombinePdf, ConvolutionPdf, DataSet, DecayInfo4, DP4Pair, Lineshape, Lineshapes, SpinFactor,
                  DaughterPair, DecayInfo3, EvalFunc, EventNumber, ExpPdf, FitManager, FitManagerMinuit2,
                  GaussianPdf, GeneralError, GooPdf, MultiPolynomialPdf, NonRes, Observable, OutOfRange, PdfBase,
                  PolynomialPdf, ProdPdf, ResonancePdf, Resonances, UnbinnedDataSet, Variable, get_precision,
                  readFromFile, readListOfNumbers, set_precision, writeToFile)
from .engine import Engine, FitResult, Minimizer

__all__ = [
    "AddPdf", "CombinePdf", "ConvolutionPdf", "DataSet", "EvalFunc", "EventNumber", "ExpPdf", "FitManager",
    "FitManagerMinuit2", "GaussianPdf", "GeneralError", "GooPdf", "Observable", "OutOfRange", "PdfBase",
    "PolynomialPdf", "ProdPdf", "UnbinnedDataSet", "Variable", "Engine", "FitResult", "Minimizer",
    "get_precision", "set_precision", "Amp3Body", "DecayInfo3", "DaughterPair", "PAIR_12", "PAIR_13", "PAIR_23",
    "ResonancePdf", "Resonances", "RBW", "NonRes", "MultiPolynomialPdf", "Amp4Body", "Amplitude", "AmpComponent",
    "DecayInfo4", "DP4Pair", "FF", "Lineshape", "Lineshapes", "SF_4Body", "SpinFactor", "BinnedDataSet",
    "FitControl", "UnbinnedNllFit", "BinnedNllFit", "BinnedErrorFit", "BinnedChisqFit", "writeToFile",
    "readFromFile", "readListOfNumbers",
]
