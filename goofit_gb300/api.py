"""GooFit-compatible host API over the GB300 engine.

Mirrors the reference's operator surface (include/goofit/Variable.h,
DataSet.h, UnbinnedDataSet.h, PdfBase.h, PDFs/GooPdf.h, PDFs/basic/*.h,
PDFs/combine/*.h, fitting/FitManagerMinuit2.h) and its Python bindings
(python/goofit/*.cpp): same class names, constructor argument orders and
method names.  A PDF object describes one node; the tree under a root PDF is
flattened depth-first (as PdfBase::populateArrays does,
src/PDFs/PdfBase.cu:268-311) into the engine's node list, and every
evaluation runs on the GPU through libgfengine.so.
"""
from __future__ import annotations

import enum
import math
import time
from typing import Iterable, Sequence

import numpy as np

from . import _abi as A
from .engine import Engine, FitResult

_DEFAULT_PRECISION = "mixed"


def set_precision(p: str) -> None:
    """Arithmetic of new engines: 'mixed' (FP32 events, FP64 reductions) or 'fp64'."""
    global _DEFAULT_PRECISION
    if p not in ("mixed", "fp64"):
        raise ValueError(p)
    _DEFAULT_PRECISION = p


def get_precision() -> str:
    return _DEFAULT_PRECISION


class GeneralError(RuntimeError):
    """GooFit::GeneralError (include/goofit/Error.h:9-19)."""


class OutOfRange(GeneralError):
    """GooFit::OutOfRange raised by DataSet::checkAllVars (src/goofit/DataSet.cpp:72-77)."""

    def __init__(self, name, value, lo, hi):
        super().__init__(f"{name} value {value} outside of range {lo} to {hi}")


class EvalFunc(enum.IntEnum):
    """include/goofit/FitControl.h:11"""
    Eval = 0
    NLL = 1
    Prob = 2
    BinAvg = 3
    BinWithError = 4
    Chisq = 5


# ---------------------------------------------------------------- variables
class Indexable:
    """Named quantity with value and limits (include/goofit/Variable.h:22-106).

    Python objects are references, so copies alias as the reference's
    shared_ptr members do."""

    def __init__(self, name: str, value: float = 0.0, lowerlimit: float = 0.0, upperlimit: float = 0.0):
        self.name = name
        self._value = float(value)
        self.lowerlimit = float(lowerlimit)
        self.upperlimit = float(upperlimit)
        self.index = -1

    @property
    def value(self) -> float:
        return self._value

    @value.setter
    def value(self, v: float) -> None:
        self._value = float(v)

    def getName(self) -> str:
        return self.name

    def getValue(self) -> float:
        return self._value

    def setValue(self, v: float) -> None:
        self._value = float(v)

    def getLowerLimit(self) -> float:
        return self.lowerlimit

    def getUpperLimit(self) -> float:
        return self.upperlimit

    def setLowerLimit(self, v: float) -> None:
        self.lowerlimit = float(v)

    def setUpperLimit(self, v: float) -> None:
        self.upperlimit = float(v)

    def getIndex(self) -> int:
        return self.index

    def setIndex(self, i: int) -> None:
        self.index = i

    def __float__(self) -> float:
        return self._value

    def __bool__(self) -> bool:
        # in range check (Variable.h:101-104)
        return self.upperlimit == self.lowerlimit or (self.lowerlimit <= self._value <= self.upperlimit)

    def __repr__(self) -> str:
        return f"{type(self).__name__}({self.name!r}, {self._value})"


class Observable(Indexable):
    """include/goofit/Variable.h:109-140 (numbins defaults to 100)."""

    def __init__(self, name: str, lowerlimit: float, upperlimit: float):
        super().__init__(name, 0.0, lowerlimit, upperlimit)
        self.numbins = 100
        self.is_event_number = False

    def setNumBins(self, n: int) -> None:
        self.numbins = int(n)

    def getNumBins(self) -> int:
        return self.numbins

    def getBinSize(self) -> float:
        return (self.upperlimit - self.lowerlimit) / self.numbins

    def isEventNumber(self) -> bool:
        return self.is_event_number


class EventNumber(Observable):
    """include/goofit/Variable.h:246-263."""
    maxint = float(1 << 53)

    def __init__(self, name: str, lowerlimit: float = 0.0, upperlimit: float = maxint):
        super().__init__(name, lowerlimit, upperlimit)
        self.is_event_number = True


class Variable(Indexable):
    """include/goofit/Variable.h:143-241; the constructors keep the reference's meanings:

    Variable(n, v)                 constant (fixed)
    Variable(n, v, err)            fixed, no limits (the reference marks it fixed)
    Variable(n, v, lo, hi)         free, limited, error 0.1 (hi - lo)
    Variable(n, v, err, lo, hi[, fixed])
    """

    def __init__(self, name: str, value: float, *args):
        if len(args) == 0:
            super().__init__(name, value, value + 0.01, value - 0.01)
            self.error, self.fixed = 0.002, True
        elif len(args) == 1:
            super().__init__(name, value, 0.0, 0.0)
            self.error, self.fixed = float(args[0]), True
        elif len(args) == 2:
            super().__init__(name, value, args[0], args[1])
            self.error, self.fixed = 0.1 * (args[1] - args[0]), False
        elif len(args) in (3, 4):
            super().__init__(name, value, args[1], args[2])
            self.error = float(args[0])
            self.fixed = bool(args[3]) if len(args) == 4 else False
        else:
            raise TypeError("Variable(name, value[, err][, lo, hi][, fixed])")
        self._blind = 0.0
        self.fitter_index = -1
        self.changed = True

    def getError(self) -> float:
        return self.error

    def setError(self, e: float) -> None:
        self.error = float(e)

    def IsFixed(self) -> bool:
        return self.fixed

    def setFixed(self, f: bool) -> None:
        self.fixed = bool(f)

    def setBlind(self, b: float) -> None:
        self._blind = float(b)

    def getFitterIndex(self) -> int:
        return self.fitter_index

    def __repr__(self) -> str:
        s = f"{self.name}: {self._value} +/- {self.error}"
        if not self.fixed:
            s += f" [{self.lowerlimit}, {self.upperlimit}]"
        return s


# ---------------------------------------------------------------- datasets
class DataSet:
    """include/goofit/DataSet.h"""

    def __init__(self, observables, name: str = ""):
        if isinstance(observables, Observable):
            observables = [observables]
        self.observables: list[Observable] = list(observables)
        self.name = name or ", ".join(o.name for o in self.observables)
        self.numEventsAdded = 0

    def getObservables(self) -> list[Observable]:
        return self.observables

    def numVariables(self) -> int:
        return len(self.observables)

    def getNumEvents(self) -> int:
        return self.numEventsAdded

    def getName(self) -> str:
        return self.name

    def indexOfVariable(self, var: Observable) -> int:
        for i, o in enumerate(self.observables):
            if o is var:
                return i
        raise GeneralError("Invalid variable access into dataset!")

    def checkAllVars(self) -> None:
        for o in self.observables:
            if not o:
                raise OutOfRange(o.name, o.value, o.lowerlimit, o.upperlimit)


class UnbinnedDataSet(DataSet):
    """include/goofit/UnbinnedDataSet.h; columns kept as float64 arrays."""

    def __init__(self, observables, name: str = ""):
        super().__init__(observables, name)
        self._chunks: list[np.ndarray] = []
        self._pending: list[list[float]] = []
        self._cache: np.ndarray | None = None
        self.version = 0

    def _touch(self) -> None:
        self._cache = None
        self.version += 1

    def addEvent(self, *values) -> None:
        if values:
            if len(values) != len(self.observables):
                raise GeneralError(f"You must pass the correct number of values ({len(self.observables)}) to addEvent")
            for o, v in zip(self.observables, values):
                o.value = v
        self.checkAllVars()
        self._pending.append([o.value for o in self.observables])
        self.numEventsAdded += 1
        self._touch()

    def _flush(self) -> None:
        if self._pending:
            self._chunks.append(np.asarray(self._pending, dtype=np.float64).T.reshape(len(self.observables), -1))
            self._pending = []

    def to_numpy(self) -> np.ndarray:
        """(n_observables, n_events) array."""
        if self._cache is None:
            self._flush()
            if self._chunks:
                self._cache = np.concatenate(self._chunks, axis=1) if len(self._chunks) > 1 else self._chunks[0]
                self._chunks = [self._cache]
            else:
                self._cache = np.zeros((len(self.observables), 0))
        return self._cache

    to_matrix = to_numpy

    def from_numpy(self, mat, filter: bool = False) -> None:
        """UnbinnedDataSet::from_matrix (include/goofit/UnbinnedDataSet.h:50-71)."""
        m = np.asarray(mat, dtype=np.float64)
        if m.ndim == 1:
            m = m.reshape(1, -1)
        nobs = len(self.observables)
        if m.shape[0] not in (nobs, nobs - 1):
            raise GeneralError(f"The wrong number of rows, expected {nobs}, but matrix had {m.shape[0]}")
        if m.shape[0] == nobs - 1:
            idx = np.arange(self.numEventsAdded, self.numEventsAdded + m.shape[1], dtype=np.float64)
            m = np.vstack([m, idx])
        ok = np.ones(m.shape[1], dtype=bool)
        for i, o in enumerate(self.observables):
            if o.upperlimit != o.lowerlimit:
                ok &= (m[i] >= o.lowerlimit) & (m[i] <= o.upperlimit)
        if filter:
            m = m[:, ok]
        elif not ok.all():
            bad = int(np.argmin(ok))
            o = next(o for i, o in enumerate(self.observables)
                     if o.upperlimit != o.lowerlimit and not (o.lowerlimit <= m[i, bad] <= o.upperlimit))
            raise OutOfRange(o.name, float(m[self.observables.index(o), bad]), o.lowerlimit, o.upperlimit)
        self._flush()
        self._chunks.append(np.ascontiguousarray(m))
        self.numEventsAdded += m.shape[1]
        self._touch()

    from_matrix = from_numpy

    def getValue(self, var: Observable, idx: int) -> float:
        if idx >= self.getNumEvents():
            raise GeneralError(f"UnbinnedDataSet: Attempted to find {var.name} in event {idx} when only "
                               f"{self.getNumEvents()} events exits")
        return float(self.to_numpy()[self.indexOfVariable(var), idx])

    def __getitem__(self, key):
        return self.to_numpy()[key]

    def loadEvent(self, idx: int) -> None:
        col = self.to_numpy()[:, idx]
        for o, v in zip(self.observables, col):
            o.value = v

    def clear(self) -> None:
        self._chunks, self._pending, self.numEventsAdded = [], [], 0
        self._touch()

    def column(self, var: Observable) -> np.ndarray:
        return self.to_numpy()[self.indexOfVariable(var)]

    def fillWithGrid(self) -> None:
        """UnbinnedDataSet::fillWithGrid (src/goofit/UnbinnedDataSet.cpp:67-105): first observable fastest."""
        if self.getNumEvents():
            raise GeneralError("The dataset must be empty to fill with grid!")
        axes = []
        for o in self.observables:
            if o.is_event_number:
                axes.append(None)
            else:
                step = (o.upperlimit - o.lowerlimit) / o.numbins
                axes.append(o.lowerlimit + (np.arange(o.numbins) + 0.5) * step)
        sizes = [len(a) for a in axes if a is not None]
        total = int(np.prod(sizes)) if sizes else 1
        cols = []
        stride = 1
        for a in axes:
            if a is None:
                cols.append(None)
                continue
            cols.append(np.tile(np.repeat(a, stride), total // (stride * len(a))))
            stride *= len(a)
        m = np.zeros((len(self.observables), total))
        for i, (o, c) in enumerate(zip(self.observables, cols)):
            m[i] = np.arange(total, dtype=np.float64) + o.value if c is None else c
        self._flush()
        self._chunks.append(m)
        self.numEventsAdded += total
        self._touch()


# ---------------------------------------------------------------- PDFs
class BinnedDataSet(DataSet):
    """include/goofit/BinnedDataSet.h, src/goofit/BinnedDataSet.cpp: counts on the observables' bin grid
    (global bin = sum local_i * prod_{j<i} nbins_j)."""

    def __init__(self, observables, name: str = ""):
        super().__init__(observables, name)
        self.binsizes = [o.getNumBins() for o in self.observables]
        self.binvalues = np.zeros(int(np.prod(self.binsizes)))
        self.binerrors: np.ndarray | None = None
        self.version = 0

    def getNumBins(self) -> int:
        return len(self.binvalues)

    def _local(self, global_bin: int) -> list[int]:
        out = []
        for n in self.binsizes:
            out.append(global_bin % n)
            global_bin //= n
        return out

    def getBinNumber(self) -> int:
        ret, prior = 0, 1
        for o, n in zip(self.observables, self.binsizes):
            b = int(np.floor((o.value - o.lowerlimit) / ((o.upperlimit - o.lowerlimit) / n)))
            ret += b * prior
            prior *= n
        return ret

    def addEvent(self) -> None:
        self.checkAllVars()
        self.binvalues[self.getBinNumber()] += 1
        self.numEventsAdded += 1
        self.version += 1

    def addWeightedEvent(self, weight: float) -> None:
        self.checkAllVars()
        self.binvalues[self.getBinNumber()] += weight
        self.numEventsAdded += 1
        self.version += 1

    def fill(self, values: np.ndarray, weights: np.ndarray | None = None) -> None:
        """Adds many events at once: values (n_obs, n) inside the observables' ranges."""
        v = np.atleast_2d(np.asarray(values, dtype=np.float64))
        g = np.zeros(v.shape[1], dtype=np.int64)
        prior = 1
        for k, (o, n) in enumerate(zip(self.observables, self.binsizes)):
            b = np.floor((v[k] - o.lowerlimit) / ((o.upperlimit - o.lowerlimit) / n)).astype(np.int64)
            g += np.clip(b, 0, n - 1) * prior
            prior *= n
        np.add.at(self.binvalues, g, 1.0 if weights is None else np.asarray(weights, dtype=np.float64))
        self.numEventsAdded += v.shape[1]
        self.version += 1

    def getBinContent(self, b: int) -> float:
        return float(self.binvalues[b])

    def setBinContent(self, b: int, value: float) -> None:
        self.binvalues[b] = value
        self.version += 1

    def getBinSize(self, ivar: int) -> float:
        o = self.observables[ivar]
        return (o.upperlimit - o.lowerlimit) / self.binsizes[ivar]

    def getBinCenter(self, var, b: int) -> float:
        ivar = var if isinstance(var, int) else self.indexOfVariable(var)
        ret = self.getBinSize(ivar)
        ret *= self._local(b)[ivar] + 0.5
        ret += self.observables[ivar].lowerlimit
        return ret

    def getBinVolume(self, b: int) -> float:
        ret = 1.0
        for i in range(len(self.observables)):
            ret *= self.getBinSize(i)
        return ret

    def getBinError(self, b: int) -> float:
        if self.binerrors is None:
            return math.sqrt(self.binvalues[b])
        return float(self.binerrors[b])

    def setBinError(self, b: int, value: float) -> None:
        # the first explicit error switches every bin to explicit errors, zero where unset (as the reference)
        if self.binerrors is None:
            self.binerrors = np.zeros_like(self.binvalues)
        self.binerrors[b] = value
        self.version += 1

    def getNumWeightedEvents(self) -> float:
        return float(self.binvalues.sum())

    def engine_columns(self, obs: list[Observable], errors: bool) -> np.ndarray:
        """Bin centres of `obs`, then contents, then volumes (or errors): PdfBase::setData's binned layout."""
        n = self.getNumBins()
        rows = []
        idx = np.arange(n)
        for o in obs:
            ivar = self.indexOfVariable(o)
            prior = int(np.prod(self.binsizes[:ivar])) if ivar else 1
            local = (idx // prior) % self.binsizes[ivar]
            rows.append(self.getBinSize(ivar) * (local + 0.5) + o.lowerlimit)
        rows.append(self.binvalues.copy())
        if errors:
            rows.append(self.binerrors.copy() if self.binerrors is not None else np.sqrt(self.binvalues))
        else:
            rows.append(np.full(n, self.getBinVolume(0)))
        return np.vstack(rows)


# ---------------------------------------------------------------- fit controls
class FitControl:
    """include/goofit/FitControl.h: which metric the fit minimises."""
    metric = A.GF_FIT_UNBINNED_NLL
    binned = False
    errors_on_bins = False

    def binnedFit(self) -> bool:
        return self.binned

    def binErrors(self) -> bool:
        return self.errors_on_bins


class UnbinnedNllFit(FitControl):
    metric = A.GF_FIT_UNBINNED_NLL


class BinnedNllFit(FitControl):
    metric, binned = A.GF_FIT_BINNED_NLL, True


class BinnedErrorFit(FitControl):
    metric, binned, errors_on_bins = A.GF_FIT_BINNED_ERROR, True, True


class BinnedChisqFit(FitControl):
    metric, binned = A.GF_FIT_BINNED_CHISQ, True


def _unique(seq: Iterable) -> list:
    out, seen = [], set()
    for x in seq:
        if id(x) not in seen:
            seen.add(id(x))
            out.append(x)
    return out


class PdfBase:
    """include/goofit/PdfBase.h: registration lists, data, normalisation, fit."""

    op: int = 0

    def __init__(self, pdf_name: str, name: str, *registered):
        self.pdf_name = pdf_name
        self.name = name
        self.parametersList: list[Variable] = []
        self.constantsList: list[float] = []
        self.observablesList: list[Observable] = []
        self.components: list[PdfBase] = []
        self.integrationBins = 0
        self.flags = 0
        self.data = None
        self.fitControl: FitControl = UnbinnedNllFit()
        self._engines: dict = {}
        for r in registered:
            if isinstance(r, Observable):
                self.registerObservable(r)
            elif isinstance(r, Variable):
                self.registerParameter(r)
            else:
                raise TypeError(r)

    # registration (src/goofit/PdfBase.cpp)
    def registerParameter(self, v: Variable) -> None:
        self.parametersList.append(v)

    def registerConstant(self, c: float) -> None:
        self.constantsList.append(float(c))

    def registerObservable(self, o: Observable) -> None:
        if all(o is not q for q in self.observablesList):
            self.observablesList.append(o)

    def getName(self) -> str:
        return self.name

    def getPdfName(self) -> str:
        return self.pdf_name

    def getParameters(self) -> list[Variable]:
        ret = list(self.parametersList)
        for c in self.components:
            ret += c.getParameters()
        return _unique(ret)

    def getObservables(self) -> list[Observable]:
        ret = list(self.observablesList)
        for c in self.components:
            ret += c.getObservables()
        return _unique(ret)

    def getComponents(self) -> list["PdfBase"]:
        return self.components

    def getParameterByName(self, n: str):
        for p in self.getParameters():
            if p.name == n:
                return p
        return None

    def setIntegrationFineness(self, i: int) -> None:
        self.integrationBins = int(i)

    def setCommonNorm(self, v: bool = True) -> None:
        self.flags = (self.flags | A.GF_FLAG_COMMON_NORM) if v else (self.flags & ~A.GF_FLAG_COMMON_NORM)

    def setSeparateNorm(self, v: bool = True) -> None:
        self.flags = (self.flags | A.GF_FLAG_SEPARATE_NORM) if v else (self.flags & ~A.GF_FLAG_SEPARATE_NORM)

    def getCommonNorm(self) -> bool:
        return bool(self.flags & A.GF_FLAG_COMMON_NORM)

    def getSeparateNorm(self) -> bool:
        return bool(self.flags & A.GF_FLAG_SEPARATE_NORM)

    def setData(self, data) -> None:
        """PdfBase::setData: a BinnedDataSet switches an unbinned fit control to BinnedNllFit
        (src/PDFs/PdfBase.cu:444-445)."""
        self.data = data
        if isinstance(data, BinnedDataSet) and not self.fitControl.binnedFit():
            self.fitControl = BinnedNllFit()

    def setFitControl(self, fc: "FitControl") -> None:
        self.fitControl = fc

    def getData(self):
        return self.data

    def copyParams(self) -> None:
        """Parameters are read from the Variables at every evaluation."""

    def _node_consts(self) -> list[float]:
        return self.constantsList

    # ---- flattening ----
    def _flatten(self):
        params = self.getParameters()
        pidx = {id(v): i for i, v in enumerate(params)}
        obs = self.getObservables()
        oidx = {id(o): i for i, o in enumerate(obs)}
        nodes: list = []

        order: list = []

        def visit(p: "PdfBase") -> int:
            i = len(nodes)
            nodes.append(None)
            order.append(p)
            kids = [visit(c) for c in p.components]
            nodes[i] = dict(op=p.op, flags=p.flags, params=[pidx[id(v)] for v in p.parametersList],
                            consts=list(p._node_consts()), obs=[oidx[id(o)] for o in p.observablesList],
                            children=kids, integration_bins=p.integrationBins)
            return i

        visit(self)
        self._flat_order = order
        return nodes, params, obs

    def _engine_setup(self, eng, node: int) -> None:
        """Per-node engine state beyond the tree (Amp4Body: its normalisation events)."""

    def _engine_for(self, data, precision: str | None = None):
        """Engine with this PDF as root and `data` uploaded; cached per (precision, data)."""
        precision = precision or _DEFAULT_PRECISION
        nodes, params, obs = self._flatten()
        nd = self._nondiff_all()
        mask = [0 if (v.fixed or id(v) in nd) else 1 for v in params]
        olist = [(o.lowerlimit, o.upperlimit, o.numbins, 1 if o.is_event_number else 0) for o in obs]
        metric = self.fitControl.metric if isinstance(data, BinnedDataSet) else A.GF_FIT_UNBINNED_NLL
        key = repr((nodes, olist, mask, metric))
        ent = self._engines.get(precision)
        if ent is None or ent["key"] != key:
            eng = ent["engine"] if ent and ent["metric"] == metric else Engine(precision)
            if metric != A.GF_FIT_UNBINNED_NLL:
                eng.set_fit_metric(metric)
            eng.set_tree(nodes, olist, len(params), mask)
            for i, p in enumerate(self._flat_order):
                p._engine_setup(eng, i)
            ent = dict(engine=eng, key=key, data=None, version=-1, metric=metric)
            self._engines[precision] = ent
        eng = ent["engine"]
        if data is not None and (ent["data"] is not data or ent["version"] != getattr(data, "version", 0)):
            if isinstance(data, BinnedDataSet):
                cols = data.engine_columns(obs, self.fitControl.binErrors())
            elif data.getNumEvents():
                cols = np.vstack([data.column(o) for o in obs])
            else:
                cols = np.zeros((len(obs), 0))
            eng.upload(cols)
            ent["data"], ent["version"] = data, getattr(data, "version", 0)
        return eng, params

    def _nondiff_params(self) -> set:
        """ids of parameters the engine provides no analytic derivative for (below this node)."""
        return set()

    def _nondiff_all(self) -> set:
        ids = set(self._nondiff_params())
        for c in self.components:
            ids |= c._nondiff_all()
        return ids

    @staticmethod
    def _param_values(params: Sequence[Variable]) -> np.ndarray:
        return np.array([v.value - v._blind for v in params], dtype=np.float64)

    def normalize(self) -> float:
        """Integral of this PDF as GooPdf::normalize returns it (src/PDFs/GooPdf.cu:340-396)."""
        data = self.data if self.data is not None else self._point_dataset()
        eng, params = self._engine_for(data)
        eng.set_params(self._param_values(params))
        I, N = eng.normalize()
        return float(I[0])

    def calculateNLL(self) -> float:
        if self.data is None:
            raise GeneralError("no data set")
        eng, params = self._engine_for(self.data)
        return eng.nll(self._param_values(params))

    def _point_dataset(self) -> UnbinnedDataSet:
        ds = UnbinnedDataSet(self.getObservables())
        ds.addEvent()
        return ds

    def fitTo(self, data, verbosity: int = 3) -> FitResult:
        old = self.data
        self.setData(data)
        try:
            return self.fit(verbosity)
        finally:
            self.setData(old)

    def fit(self, verbosity: int = 3) -> FitResult:
        fm = FitManager(self)
        fm.verbosity = verbosity
        return fm.fit()


class GooPdf(PdfBase):
    """include/goofit/PDFs/GooPdf.h"""

    def integrate(self, lo: float, hi: float) -> float:
        return 0.0

    def hasAnalyticIntegral(self) -> bool:
        return False

    def makeGrid(self) -> UnbinnedDataSet:
        grid = UnbinnedDataSet(self.getObservables())
        grid.fillWithGrid()
        return grid

    def _probs(self, data, metric=A.GF_METRIC_PROB) -> np.ndarray:
        eng, params = self._engine_for(data)
        eng.set_params(self._param_values(params))
        return eng.eval_events(metric)

    def getValue(self, evalfunc: EvalFunc = EvalFunc.Eval) -> float:
        """GooPdf::getValue (src/PDFs/GooPdf.cu:214-248) at the observables' current values."""
        metric = {EvalFunc.Prob: A.GF_METRIC_PROB, EvalFunc.Eval: A.GF_METRIC_EVAL,
                  EvalFunc.NLL: A.GF_METRIC_NLL}.get(evalfunc)
        if metric is None:
            raise GeneralError("That EvalFunc is not supported")
        return float(self._probs(self._point_dataset(), metric)[0])

    def evaluateAtPoints(self, var: Observable) -> list[float]:
        """GooPdf::evaluateAtPoints (src/PDFs/GooPdf.cu:187-212): normalised values at var's bin centres."""
        ds = UnbinnedDataSet(self.getObservables())
        step = var.getBinSize()
        saved = var.value
        for i in range(var.getNumBins()):
            var.value = var.lowerlimit + (i + 0.5) * step
            ds.addEvent()
        var.value = saved
        return list(self._probs(ds, A.GF_METRIC_PROB))

    def getCompProbsAtDataPoints(self) -> list[list[float]]:
        """GooPdf::getCompProbsAtDataPoints (src/PDFs/GooPdf.cu:402-435)."""
        if self.data is None:
            raise GeneralError("no data set")
        out = [list(self._probs(self.data))]
        for c in self.components:
            sub = UnbinnedDataSet(c.getObservables())
            sub.from_numpy(np.vstack([self.data.column(o) for o in c.getObservables()]))
            out.append(list(c._probs(sub)))
        return out

    def scan(self, var: Variable, values: list | None = None) -> list[float]:
        """GooPdf::scan (src/PDFs/GooPdf.cpp:69-82): NLL at bin centres of a parameter."""
        res = []
        step = (var.upperlimit - var.lowerlimit) / 100
        v = var.lowerlimit + 0.5 * step
        saved = var.value
        while v < var.upperlimit:
            var.value = v
            res.append(self.calculateNLL())
            v += step
        var.value = saved
        if values is not None:
            values[:] = res
        return res

    def fillMCDataSimple(self, events: int, seed: int = 0) -> None:
        """PdfBase::fillMCDataSimple (src/goofit/PdfBase.cpp:154-203): inverse-CDF fill of the data set."""
        obs = self.getObservables()
        if len(obs) != 1:
            raise GeneralError("You can only fill MC on a 1D dataset with a simple fill")
        var = obs[0]
        origdata = self.data
        if origdata is None:
            raise GeneralError("Can't run on a PDF with no DataSet to fill!")
        grid = UnbinnedDataSet(var)
        grid.fillWithGrid()
        pdfValues = np.asarray(self._probs(grid))
        rng = np.random.default_rng(seed if seed else None)
        integral = np.cumsum(pdfValues)
        integral /= integral[-1]
        r = rng.random(events)
        j = np.searchsorted(integral, r, side="left")
        x = grid.column(var)[j] + var.getBinSize() * (rng.random(events) - 0.5)
        x = np.clip(x, var.lowerlimit, var.upperlimit)
        origdata.from_numpy(x.reshape(1, -1))


class CombinePdf(GooPdf):
    """include/goofit/PDFs/CombinePdf.h"""


class ExpPdf(GooPdf):
    """include/goofit/PDFs/basic/ExpPdf.h, src/PDFs/basic/ExpPdf.cu"""

    def __init__(self, name: str, x: Observable, alpha, offset: Variable | None = None):
        if isinstance(alpha, (list, tuple)):
            if not alpha:
                raise GeneralError("Weights are empty!")
            if offset is None:
                super().__init__("ExpPdf", name, x)
                self.op = A.GF_OP_EXP_POLY
            else:
                super().__init__("ExpPdf", name, x, offset)
                self.op = A.GF_OP_EXP_POLY_OFFSET
            for w in alpha:
                self.registerParameter(w)
        elif offset is None:
            super().__init__("ExpPdf", name, x, alpha)
            self.op = A.GF_OP_EXP
        else:
            super().__init__("ExpPdf", name, x, offset, alpha)
            self.op = A.GF_OP_EXP_OFFSET

    def hasAnalyticIntegral(self) -> bool:
        return len(self.parametersList) == 1

    def integrate(self, lo: float, hi: float) -> float:
        alpha = self.parametersList[0].value
        if alpha == 0:
            return hi - lo
        return (math.exp(alpha * hi) - math.exp(alpha * lo)) / alpha


class GaussianPdf(GooPdf):
    """include/goofit/PDFs/basic/GaussianPdf.h"""
    op = A.GF_OP_GAUSSIAN

    def __init__(self, name: str, x: Observable, mean: Variable, sigma: Variable):
        super().__init__("GaussianPdf", name, x, mean, sigma)

    def hasAnalyticIntegral(self) -> bool:
        return True

    def integrate(self, lo: float, hi: float) -> float:
        return self.parametersList[1].value * math.sqrt(2.0) * math.sqrt(math.atan2(0.0, -1.0))


class PolynomialPdf(GooPdf):
    """include/goofit/PDFs/basic/PolynomialPdf.h (one-observable forms)."""

    def __new__(cls, name: str, x, *args, **kw):
        if cls is PolynomialPdf and isinstance(x, (list, tuple)):
            return MultiPolynomialPdf(name, x, *args, **kw)
        return super().__new__(cls)

    def __init__(self, name: str, x: Observable, weights: Sequence[Variable], *args):
        super().__init__("PolynomialPdf", name, x)
        x0 = None
        lowest = 0
        if args and isinstance(args[0], Variable):
            x0 = args[0]
            lowest = int(args[1]) if len(args) > 1 else 0
        elif args:
            lowest = int(args[0])
        self.registerConstant(lowest)
        for w in weights:
            self.registerParameter(w)
        if x0 is not None:
            self.registerParameter(x0)
            self.op = A.GF_OP_POLYNOMIAL_OFFSET
        else:
            self.op = A.GF_OP_POLYNOMIAL


class AddPdf(CombinePdf):
    """include/goofit/PDFs/combine/AddPdf.h: AddPdf(name, weights, comps) / AddPdf(name, frac, pdf1, pdf2)."""

    def __init__(self, name: str, weights, comps, third=None):
        super().__init__("AddPdf", name)
        if isinstance(weights, Variable):
            comps_l = [comps, third]
            ws = [weights]
            self.extended = False
        else:
            ws, comps_l = list(weights), list(comps)
            if len(ws) != len(comps_l) and len(ws) + 1 != len(comps_l):
                raise GeneralError(f"Size of weights {len(ws)} (+1) != comps {len(comps_l)}")
            self.extended = len(ws) == len(comps_l)
        for c in comps_l:
            if c is None:
                raise GeneralError("Invalid component")
            self.components.append(c)
        self.observablesList = self.getObservables()
        for w in ws:
            self.registerParameter(w)
        self.op = A.GF_OP_ADD_EXT if self.extended else A.GF_OP_ADD


class ProdPdf(CombinePdf):
    """include/goofit/PDFs/combine/ProdPdf.h"""
    op = A.GF_OP_PROD

    def __init__(self, name: str, comps: Sequence[PdfBase]):
        super().__init__("ProdPdf", name)
        self.components = list(comps)
        self.observablesList = self.getObservables()
        self.registerConstant(len(self.components))


class ConvolutionPdf(CombinePdf):
    """include/goofit/PDFs/combine/ConvolutionPdf.h; integration constants default to (-10, 10, 0.01)."""
    op = A.GF_OP_CONVOLUTION
    _count = 0

    def __init__(self, name: str, x: Observable, model: GooPdf, resolution: GooPdf, numOthers: int | None = None):
        super().__init__("ConvolutionPdf", name, x)
        self.model, self.resolution = model, resolution
        self.components = [model, resolution]
        self.observablesList = self.getObservables()
        self.workSpaceIndex = ConvolutionPdf._count
        ConvolutionPdf._count += 1
        self.constantsList = [-10.0, 10.0, 0.01, float(self.workSpaceIndex)]

    def setIntegrationConstants(self, lo: float, hi: float, step: float) -> None:
        self.constantsList[0:3] = [float(lo), float(hi), float(step)]


class MultiPolynomialPdf(GooPdf):
    """Multivariate form of PolynomialPdf (src/PDFs/basic/PolynomialPdf.cu:154-207): offsets, then the
    C(maxDegree + n, n) coefficients of the monomials of total degree <= maxDegree; missing coefficients
    and offsets are padded with constants at zero, as the reference does."""
    op = A.GF_OP_MULTIPOLYNOMIAL

    def __init__(self, name: str, obses: Sequence[Observable], coeffs: Sequence[Variable],
                 offsets: Sequence[Variable] = (), maxDegree: int = 1):
        super().__init__("PolynomialPdf", name)
        self.registerConstant(maxDegree)
        npar = 1
        for i, o in enumerate(obses):
            self.registerObservable(o)
            npar *= maxDegree + 1 + i
            self.registerConstant(maxDegree + 1 + i)
        for i in range(len(self.observablesList), 1, -1):
            npar //= i
        coeffs, offsets = list(coeffs), list(offsets)
        while npar > len(coeffs):
            coeffs.append(Variable(f"{name}_extra_coeff_{len(coeffs)}", 0))
        while len(offsets) < len(obses):
            offsets.append(Variable(f"{name}_extra_offset_{len(offsets)}", 0))
        for v in offsets:
            self.registerParameter(v)
        for v in coeffs:
            self.registerParameter(v)


# ---------------------------------------------------------------- Dalitz plots
class DaughterPair(enum.IntEnum):
    """include/goofit/PDFs/physics/DalitzPlotHelpers.h: the resonance's daughter pair (cyclic index)."""
    PAIR_12 = 0
    PAIR_13 = 1
    PAIR_23 = 2


PAIR_12, PAIR_13, PAIR_23 = DaughterPair.PAIR_12, DaughterPair.PAIR_13, DaughterPair.PAIR_23


class DecayInfo3:
    """include/goofit/PDFs/physics/DalitzPlotHelpers.h:88-97.  mother_meson_radius defaults to 0 (the
    reference leaves it uninitialised)."""

    def __init__(self):
        self.motherMass = 0.0
        self.daug1Mass = 0.0
        self.daug2Mass = 0.0
        self.daug3Mass = 0.0
        self.meson_radius = 0.0
        self.mother_meson_radius = 0.0
        self.resonances: list[ResonancePdf] = []

    def add_resonance(self, r: "ResonancePdf") -> None:
        self.resonances.append(r)


class ResonancePdf(GooPdf):
    """include/goofit/PDFs/physics/resonances/Resonance.h: a resonance carries its complex coefficient
    (registered on the Amp3Body) and its own line-shape parameters."""

    def __init__(self, pdf_name: str, name: str, ar: Variable, ai: Variable):
        super().__init__(pdf_name, name)
        self.amp_real, self.amp_imag = ar, ai

    def setParameterConstantness(self, constant: bool = True) -> None:
        for v in self.parametersList:
            v.setFixed(constant)


class RBW(ResonancePdf):
    """Resonances::RBW (src/PDFs/physics/resonances/RBW.cu:93-114)."""
    op = A.GF_OP_RES_RBW

    def __init__(self, name: str, ar: Variable, ai: Variable, mass: Variable, width: Variable, sp: int, cyc: int,
                 norm: bool = True, sym: bool = False):
        super().__init__("RBW", name, ar, ai)
        self.registerParameter(mass)
        self.registerParameter(width)
        self.registerConstant(int(sp))
        self.registerConstant(int(cyc))
        self.registerConstant(1 if norm else 0)
        self.registerConstant(1 if sym else 0)


class NonRes(ResonancePdf):
    """Resonances::NonRes (src/PDFs/physics/resonances/NonRes.cu:8-20): constant amplitude 1."""
    op = A.GF_OP_RES_NONRES

    def __init__(self, name: str, ar: Variable, ai: Variable):
        super().__init__("NonRes", name, ar, ai)


class Resonances:
    """Namespace of the resonance shapes (GooFit::Resonances)."""
    RBW = RBW
    NonRes = NonRes


def _generate_sig(pdf: "GooPdf", particles: np.ndarray, columns: np.ndarray, rng: np.random.Generator):
    """Weights and accept-reject flags of phase-space events for an amplitude PDF: the weight of an event is
    the PDF's unnormalised value (|sum c A|^2 times the efficiency; the FP64 engine), flagged accepted with
    probability weight / max weight (Amp3BodyBase::fillMCFlags, src/PDFs/physics/Amp3BodyBase.cu:13-21).
    The phase-space events are flat already (unweighted), so their own weight is 1."""
    from .engine import Engine
    nodes, params, obs = pdf._flatten()
    eng = Engine("fp64")
    try:
        eng.set_tree(nodes, [(o.lowerlimit, o.upperlimit, o.numbins, int(o.is_event_number)) for o in obs],
                     len(params), [0] * len(params))
        for i, p in enumerate(pdf._flat_order):
            p._engine_setup(eng, i)
        eng.upload(np.ascontiguousarray(columns, dtype=np.float64))
        eng.set_params(np.array([v.value for v in params]))
        weights = eng.eval_events(A.GF_METRIC_EVAL)
    finally:
        eng.close()
    wmax = float(weights.max()) if weights.size else 0.0
    flags = rng.random(weights.size) * wmax < weights
    return [particles[:, i, :].copy() for i in range(particles.shape[1])], weights, flags


def _generator(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(seed)) if seed else np.random.default_rng()


class Amp3Body(GooPdf):
    """include/goofit/PDFs/physics/Amp3Body.h, src/PDFs/physics/Amp3Body.cu:127-196: coherent sum of
    resonances times an efficiency, normalised over the m12 x m13 bin grid of the two observables.

    Without an efficiency a constant one (degree-0 MultiPolynomialPdf at 1) is used."""
    op = A.GF_OP_AMP3BODY
    cacheCount = 0

    def __init__(self, name: str, m12: Observable, m13: Observable, eventNumber: EventNumber, decay: DecayInfo3,
                 eff: GooPdf | None = None):
        super().__init__("Amp3Body", name, m12, m13, eventNumber)
        self.decayInfo = decay
        self._m12, self._m13, self._eventNumber = m12, m13, eventNumber
        if eff is None:
            eff = MultiPolynomialPdf(f"{name}_constantEff", [m12, m13], [Variable(f"{name}_constantOne", 1)],
                                     [Variable(f"{name}_zero0", 0), Variable(f"{name}_zero1", 0)], 0)
        self.efficiency = eff
        self.registerConstant(len(decay.resonances))
        self.cacheToUse = Amp3Body.cacheCount
        Amp3Body.cacheCount += 1
        self.registerConstant(self.cacheToUse)
        for c in (decay.motherMass, decay.daug1Mass, decay.daug2Mass, decay.daug3Mass, decay.meson_radius,
                  decay.mother_meson_radius):
            self.registerConstant(c)
        for r in decay.resonances:
            self.registerParameter(r.amp_real)
            self.registerParameter(r.amp_imag)
            self.components.append(r)
        self.components.append(eff)
        self.setSeparateNorm()

    @staticmethod
    def resetCacheCounter() -> None:
        Amp3Body.cacheCount = 0

    def getDecayInfo(self) -> DecayInfo3:
        return self.decayInfo

    def setDataSize(self, dataSize: int, evtSize: int = 3, offset: int = 0) -> None:
        """The amplitude cache is sized by the uploaded data; kept for interface compatibility."""
        if evtSize < 3:
            raise GeneralError(f"totalEventSize {evtSize} must be 3 or more")

    def setForceIntegrals(self, f: bool = True) -> None:
        """Integrals are rebuilt whenever a resonance or efficiency parameter changes."""

    def _nondiff_params(self) -> set:
        """The efficiency's parameters (the resonance parameters have analytic derivatives)."""
        return {id(v) for v in self.efficiency.getParameters()}

    def _node_index(self) -> int:
        return 0

    def _root_engine(self):
        if self.data is None:
            raise GeneralError("no data set")
        eng, params = self._engine_for(self.data)
        eng.set_params(self._param_values(params))
        return eng

    def getCachedWave(self, i: int) -> np.ndarray:
        """Amplitude of resonance i at every data event (Amp3Body::getCachedWave)."""
        return self._root_engine().amp3_cached_wave(self._node_index(), i)

    def sumCachedWave(self, i: int) -> complex:
        return complex(self.getCachedWave(i).sum())

    def integrals(self) -> np.ndarray:
        """The n x n normalisation integrals I_ij the engine caches (before the bin size factor)."""
        return self._root_engine().amp3_integrals(self._node_index(), len(self.decayInfo.resonances))

    def GenerateSig(self, numEvents: int, seed: int = 0):
        """Amp3Body::GenerateSig (src/PDFs/physics/Amp3Body.cu:430-547): numEvents flat phase-space events of
        the decay, their invariant masses, weights (the amplitude density) and accept-reject flags.  Returns
        (particles, variables, weights, flags): three (n, 4) arrays of daughter 4-vectors (px, py, pz, E) in
        the parent frame, [m12^2, m23^2, m13^2] (the reference's VarSet order), and two length-n arrays."""
        from . import phasespace
        d = self.decayInfo
        rng = _generator(seed)
        p = phasespace.generate(d.motherMass, [d.daug1Mass, d.daug2Mass, d.daug3Mass], int(numEvents), rng)

        def m2(a, b):
            q = p[:, a] + p[:, b]
            return q[:, 3] ** 2 - np.sum(q[:, :3] ** 2, axis=1)

        m12, m13, m23 = m2(0, 1), m2(0, 2), m2(1, 2)
        cols = np.vstack([m12, m13, np.arange(len(m12), dtype=np.float64)])
        parts, w, f = _generate_sig(self, p, cols, rng)
        return parts, [m12, m23, m13], w, f

    def fit_fractions(self) -> list[list[float]]:
        """Amp3Body::fit_fractions (src/PDFs/physics/Amp3Body.cu:376-427): from the data-event caches."""
        n = len(self.decayInfo.resonances)
        eng = self._root_engine()
        waves = [eng.amp3_cached_wave(self._node_index(), i) for i in range(n)]
        coefs = [complex(r.amp_real.value, r.amp_imag.value) for r in self.decayInfo.resonances]
        ne = len(waves[0])
        amps = [[0.0] * n for _ in range(n)]
        total = 0.0
        for i in range(n):
            for j in range(n):
                b = float(np.sum((coefs[i] * np.conj(coefs[j]) * waves[i] * np.conj(waves[j])).real))
                total += b
                amps[i][j] = b / ne
        total /= ne
        return [[amps[i][j] / total for j in range(n)] for i in range(n)]


# ---------------------------------------------------------------- 4-body amplitudes
class SF_4Body(enum.IntEnum):
    """include/goofit/PDFs/physics/SpinFactors.h:18-35"""
    DtoPP1_PtoSP2_StoP3P4 = 0
    DtoPP1_PtoVP2_VtoP3P4 = 1
    DtoV1V2_V1toP1P2_V2toP3P4_S = 2
    DtoV1V2_V1toP1P2_V2toP3P4_P = 3
    DtoV1V2_V1toP1P2_V2toP3P4_D = 4
    DtoAP1_AtoVP2_VtoP3P4 = 5
    DtoAP1_AtoVP2Dwave_VtoP3P4 = 6
    DtoVS_VtoP1P2_StoP3P4 = 7
    DtoV1P1_V1toV2P2_V2toP3P4 = 8
    DtoAP1_AtoSP2_StoP3P4 = 9
    DtoTP1_TtoVP2_VtoP3P4 = 10
    FF_12_34_L1 = 11
    FF_12_34_L2 = 12
    FF_123_4_L1 = 13
    FF_123_4_L2 = 14
    ONE = 15


class FF(enum.IntEnum):
    """Form factors of a line shape (include/goofit/PDFs/physics/lineshapes/Lineshape.h:18)."""
    One = 0
    BL = 1
    BL_Prime = 2
    BL2 = 3


class DP4Pair(enum.IntEnum):
    """Daughter combinations of a 4-body line shape (include/goofit/PDFs/physics/DalitzPlotHelpers.h:58-77)."""
    M_12 = 0
    M_34 = 1
    M_13 = 2
    M_14 = 3
    M_23 = 4
    M_24 = 5
    M_12_3 = 6
    M_13_2 = 7
    M_23_1 = 8
    M_12_4 = 9
    M_14_2 = 10
    M_24_1 = 11
    M_13_4 = 12
    M_14_3 = 13
    M_34_1 = 14
    M_23_4 = 15
    M_24_3 = 16
    M_34_2 = 17


for _p in DP4Pair:
    globals()[_p.name] = _p


class AmpComponent(GooPdf):
    """include/goofit/PDFs/physics/AmpComponent.h: a building block of a 4-body amplitude."""


class SpinFactor(AmpComponent):
    """SpinFactor(name, SF, mD0, P0, P1, P2, P3) (src/PDFs/physics/SpinFactors.cu:586-664)."""
    op = A.GF_OP_SPINFACTOR

    def __init__(self, name: str, SF: SF_4Body, mD0: float, P0: int, P1: int, P2: int, P3: int):
        super().__init__("SpinFactor", name)
        self._SF, self._P = SF_4Body(SF), (P0, P1, P2, P3)
        for c in (int(SF), mD0, P0, P1, P2, P3):
            self.registerConstant(c)


class Lineshape(AmpComponent):
    """include/goofit/PDFs/physics/lineshapes/Lineshape.h: a line shape of a daughter combination."""

    def __init__(self, pdf_name: str, name: str, mass: Variable, width: Variable, L: int, Mpair: int,
                 FormFac: FF = FF.BL_Prime, radius: float = 1.5):
        super().__init__("Lineshapes::" + pdf_name, name)
        self._L, self._Mpair, self._FormFac, self._radius = int(L), int(Mpair), FF(FormFac), float(radius)
        self.registerParameter(mass)
        self.registerParameter(width)
        for c in (int(Mpair), int(L), int(FormFac), float(radius)):
            self.registerConstant(c)

    def setParameterConstantness(self, constant: bool = True) -> None:
        for v in self.parametersList:
            v.setFixed(constant)


class _RBWLineshape(Lineshape):
    """Lineshapes::RBW (src/PDFs/physics/lineshapes/BW.cu:14-68, 136-151): mass-dependent width."""
    op = A.GF_OP_LS_RBW

    def __init__(self, name, mass, width, L, Mpair, FormFac=FF.BL_Prime, radius=1.5):
        super().__init__("RBW", name, mass, width, L, Mpair, FormFac, radius)


class _SBWLineshape(Lineshape):
    """Lineshapes::SBW (src/PDFs/physics/lineshapes/BW.cu:70-110, 155-170): constant width."""
    op = A.GF_OP_LS_SBW

    def __init__(self, name, mass, width, L, Mpair, FormFac=FF.BL_Prime, radius=1.5):
        super().__init__("SBW", name, mass, width, L, Mpair, FormFac, radius)


class Lineshapes:
    """Namespace of the 4-body line shapes (GooFit::Lineshapes); RBW and SBW are provided."""
    RBW = _RBWLineshape
    SBW = _SBWLineshape


class Amplitude(AmpComponent):
    """Amplitude(uniqueDecayStr, ar, ai, LS, SF, nPerm) (src/PDFs/physics/Amplitude.cu:11-31): the sum over
    nPerm permutations of products of its line shapes and spin factors, divided by sqrt(nPerm)."""
    op = A.GF_OP_AMPLITUDE

    def __init__(self, uniqueDecayStr: str, ar: Variable, ai: Variable, LS: Sequence[Lineshape],
                 SF: Sequence[SpinFactor], nPerm: int = 1):
        super().__init__("Amplitude", uniqueDecayStr)
        self._uniqueDecayStr = uniqueDecayStr
        self._ar, self._ai = ar, ai
        self._LS, self._SF, self._nPerm = list(LS), list(SF), int(nPerm)
        if len(self._LS) % self._nPerm or len(self._SF) % self._nPerm:
            raise GeneralError("line shape and spin factor counts must be multiples of nPerm")
        self.components = self._LS + self._SF
        for c in (self._nPerm, len(self._LS), len(self._SF)):
            self.registerConstant(c)

    def getLineShapes(self) -> list:
        return self._LS

    def getSpinFactors(self) -> list:
        return self._SF


class DecayInfo4:
    """include/goofit/PDFs/physics/DalitzPlotHelpers.h:114-120: particle_masses = [M, m1, m2, m3, m4]."""

    def __init__(self):
        self.particle_masses: list[float] = []
        self.meson_radius = 1.5
        self.amplitudes: list[Amplitude] = []
        self.amplitudes_B: list[Amplitude] = []


class Amp4Body(GooPdf):
    """Amp4Body(name, observables, decay, eff, MCeventsNorm) (src/PDFs/physics/Amp4Body.cu:94-292):
    |sum_a c_a A_a|^2 * efficiency over (m12, m34, cos12, cos34, phi[, eventNumber]), normalised by the mean
    of |sum_a c_a A_a|^2 over flat phase-space events.  The normalisation events are generated here
    (MCeventsNorm of them kept after unweighting, seeded by norm_seed); the reference draws them with
    MCBooster and keeps the accepted part of MCeventsNorm."""
    op = A.GF_OP_AMP4BODY
    cacheCount = 0

    def __init__(self, name: str, observables: Sequence[Observable], decay: DecayInfo4, eff: GooPdf | None = None,
                 MCeventsNorm: int = 5_000_000, norm_seed: int = 4242):
        from . import phasespace
        super().__init__("Amp4Body", name)
        obs = list(observables)
        if len(obs) < 5:
            raise GeneralError("Amp4Body needs the observables m12, m34, cos12, cos34, phi (and eventNumber)")
        for o in obs:
            self.registerObservable(o)
        self.decayInfo = decay
        masses = list(decay.particle_masses)
        if len(masses) != 5:
            raise GeneralError("DecayInfo4.particle_masses must hold the parent and four daughter masses")
        for m in masses:
            self.registerConstant(m)
        self.cacheToUse = Amp4Body.cacheCount
        Amp4Body.cacheCount += 1
        self.registerConstant(self.cacheToUse)
        for amp in decay.amplitudes:
            self.registerParameter(amp._ar)
            self.registerParameter(amp._ai)
            self.components.append(amp)
        if eff is None:
            eff = MultiPolynomialPdf(f"{name}_constantEff", obs[:2], [Variable(f"{name}_constantOne", 1)],
                                     [Variable(f"{name}_zero0", 0), Variable(f"{name}_zero1", 0)], 0)
        self.efficiency = eff
        self.components.append(eff)
        self.MCevents = int(MCeventsNorm)
        self.norm_events = phasespace.norm_events(masses[0], masses[1:], self.MCevents, norm_seed)
        self.setSeparateNorm()

    def _engine_setup(self, eng, node: int) -> None:
        eng.set_norm_events(node, self.norm_events)

    def _nondiff_params(self) -> set:
        """The efficiency's parameters (the line-shape parameters have analytic derivatives)."""
        return {id(v) for v in self.efficiency.getParameters()}

    def setDataSize(self, dataSize: int, evtSize: int = 6) -> None:
        """The amplitude cache is sized by the uploaded data; kept for interface compatibility."""
        if evtSize < 3:
            raise GeneralError(f"totalEventSize {evtSize} should be 3 or more")

    def setForceIntegrals(self, f: bool = True) -> None:
        """Caches are rebuilt whenever a line-shape parameter changes."""

    def _root_engine(self):
        if self.data is None:
            raise GeneralError("no data set")
        eng, params = self._engine_for(self.data)
        eng.set_params(self._param_values(params))
        return eng

    def GenerateSig(self, numEvents: int, seed: int = 0):
        """Amp4Body::GenerateSig (src/PDFs/physics/Amp4Body.cu:560-677): numEvents flat phase-space events,
        their Dim5 variables, weights (the amplitude density) and accept-reject flags.  Returns (particles,
        variables, weights, flags): four (n, 4) arrays of daughter 4-vectors (px, py, pz, E),
        [m12, m34, cos12, cos34, phi], and two length-n arrays."""
        from . import phasespace
        masses = list(self.decayInfo.particle_masses)
        rng = _generator(seed)
        p = phasespace.generate(masses[0], masses[1:], int(numEvents), rng)
        v5 = phasespace.dim5(p)
        cols = np.vstack([v5, np.arange(v5.shape[1], dtype=np.float64)])
        nobs = len(self._flatten()[2])
        parts, w, f = _generate_sig(self, p, cols[:nobs], rng)
        return parts, [v5[i] for i in range(5)], w, f

    def getCachedAmplitude(self, i: int) -> np.ndarray:
        """Amplitude i at every data event (the reference's cachedAMPs column)."""
        return self._root_engine().amp3_cached_wave(0, i)

    def normalisation_sums(self) -> np.ndarray:
        """G_ab = sum over the normalisation events of A_a conj(A_b)."""
        return self._root_engine().amp3_integrals(0, len(self.decayInfo.amplitudes))


# ---------------------------------------------------------------- fitting
class FitManager:
    """FitManagerMinuit2 surface (include/goofit/fitting/FitManagerMinuit2.h) on the project MIGRAD.

    Extra keywords: precision ('mixed'/'fp64'), gradient ('analytic' or
    'numerical', the latter is MINUIT's 2-point scheme like the reference's
    Minuit2 default) and tolerance (MnMigrad tolerance; EDM < 0.002 tol up)."""

    Valid, NotRun, InValid = 0, 50, 51

    def __init__(self, pdf: PdfBase, precision: str | None = None, gradient: str = "analytic",
                 tolerance: float = 0.1):
        self.pdf = pdf
        self.precision = precision
        self.gradient = gradient
        self.tolerance = tolerance
        self.verbosity = 3
        self.max_calls = 0
        self.strategy = 1
        self.retval = FitManager.NotRun
        self.minos = False
        self.result: FitResult | None = None
        self.wall_seconds = 0.0

    def setMaxCalls(self, n: int = 0) -> None:
        self.max_calls = int(n)

    def setVerbosity(self, v: int) -> None:
        self.verbosity = v

    def getVerbosity(self) -> int:
        return self.verbosity

    def setStrategy(self, s: int) -> None:
        self.strategy = int(s)

    def setMinos(self, flag: bool = True) -> None:
        """Asymmetric MINOS errors after the fit (FitManagerMinuit2, src/goofit/FitManagerMinuit2.cpp:58-80)."""
        self.minos = bool(flag)

    def fit(self) -> FitResult:
        pdf = self.pdf
        if pdf.data is None:
            raise GeneralError("no data set")
        eng, params = pdf._engine_for(pdf.data, self.precision)
        n = len(params)
        blind = np.array([v._blind for v in params])
        x0 = np.array([v.value for v in params]) - blind
        err = np.array([v.error for v in params])
        lo = np.array([v.lowerlimit for v in params]) - blind
        hi = np.array([v.upperlimit for v in params]) - blind
        fixed = np.array([1 if v.fixed else 0 for v in params], dtype=np.int32)
        limited = np.array([0 if (v.fixed or v.lowerlimit == v.upperlimit) else 1 for v in params], dtype=np.int32)
        for i, v in enumerate(params):
            v.fitter_index = i
        nd = pdf._nondiff_all()
        use_grad = self.gradient == "analytic" and not any(id(v) in nd for v in params if not v.fixed)
        self.used_gradient = "analytic" if use_grad else "numerical"
        t0 = time.perf_counter()
        res = eng.fit(x0, err, lo, hi, limited, fixed, tolerance=self.tolerance, strategy=self.strategy,
                      maxfcn=self.max_calls, use_grad=use_grad)
        self.wall_seconds = time.perf_counter() - t0
        for i, v in enumerate(params):
            v.value = res.values[i] + blind[i]
            v.error = res.errors[i]
        self.result = res
        # external covariance of the final Hesse over all parameters (fixed ones have zero rows)
        self.covariance = res.covariance
        self.retval = FitManager.Valid if res.valid else FitManager.InValid
        self.minos_errors = {}
        if self.minos and res.valid:
            up = 0.5
            for i, v in enumerate(params):
                if v.fixed:
                    continue
                lohi = [self._minos_side(eng, res, i, sgn, err, lo, hi, limited, fixed, use_grad, up)
                        for sgn in (-1.0, 1.0)]
                v.minos_error = (lohi[0], lohi[1])
                self.minos_errors[v.name] = v.minos_error
        if self.verbosity > 0:
            print(f"MIGRAD {'valid' if res.valid else 'INVALID'}: fmin={res.fmin:.10g} edm={res.edm:.3g} "
                  f"nfcn={res.nfcn} ({self.wall_seconds:.4f} s)")
            for v in params:
                print("  ", v, f"MINOS {v.minos_error}" if getattr(v, "minos_error", None) else "")
        return res

    def _minos_side(self, eng, res, i, sgn, err, lo, hi, limited, fixed, use_grad, up) -> float:
        """Signed MINOS error of parameter i on one side: the offset d at which min over the other free
        parameters of NLL(x_i = best + d) - fmin = up (F. James, MINUIT's MINOS; the reference runs
        Minuit2's MnMinos).  Each trial is a MIGRAD fit with x_i fixed, started at the best point; the
        offset is updated by d <- d sqrt(up / delta), exact for a parabolic profile, until delta is within
        1% of up.  A parameter limit stops the search there."""
        best = np.array(res.values)
        sig = res.errors[i] if res.errors[i] > 0 else max(abs(err[i]), 1e-12)
        fx = fixed.copy()
        fx[i] = 1
        d = sig
        for _ in range(12):
            x = best.copy()
            x[i] = best[i] + sgn * d
            at_limit = False
            if limited[i] and lo[i] < hi[i]:
                if x[i] <= lo[i] or x[i] >= hi[i]:
                    x[i] = min(max(x[i], lo[i]), hi[i])
                    at_limit = True
            r = eng.fit(x, err, lo, hi, limited, fx, tolerance=self.tolerance, strategy=self.strategy,
                        maxfcn=self.max_calls, use_grad=use_grad)
            delta = r.fmin - res.fmin
            if at_limit and delta < up:
                return float(x[i] - best[i])
            if not np.isfinite(delta) or delta <= 0:
                d *= 2.0
                continue
            if abs(delta - up) < 0.01 * up:
                return float(x[i] - best[i])
            d *= float(np.sqrt(up / delta))
        return float(sgn * d)

    def __bool__(self) -> bool:
        return self.retval == FitManager.Valid

    def __int__(self) -> int:
        return self.retval


FitManagerMinuit2 = FitManager


# ---------------------------------------------------------------- parameter files
def writeToFile(pdf: PdfBase, fname: str) -> None:
    """writeToFile (src/goofit/FunctorWriter.cpp:9-21): one line per parameter of the PDF,
    `name value error lower upper`.  Values are written with 17 significant digits (the reference streams
    them at the default 6), so that a file read back restores the parameters exactly."""
    with open(fname, "w") as w:
        for v in pdf.getParameters():
            w.write(f"{v.getName()} {v.value:.17g} {v.error:.17g} {v.lowerlimit:.17g} {v.upperlimit:.17g}\n")


def readFromFile(pdf: PdfBase, fname: str) -> None:
    """readFromFile (src/goofit/FunctorWriter.cpp:23-62): for every line whose first token names a
    parameter of the PDF, set its value, error and limits from the next four numbers; other lines are
    skipped; reading stops once every parameter has been set."""
    byname = {v.getName(): v for v in pdf.getParameters()}
    done = set()
    with open(fname) as r:
        for line in r:
            tok = line.split()
            if not tok or tok[0] not in byname:
                continue
            v = byname[tok[0]]
            value, error, lower, upper = (float(t) for t in tok[1:5])
            v.setValue(value)
            v.setError(error)
            v.setLowerLimit(lower)
            v.setUpperLimit(upper)
            done.add(tok[0])
            if len(done) == len(byname):
                break


def readListOfNumbers(fname: str) -> list[float]:
    """readListOfNumbers (src/goofit/FunctorWriter.cpp:64-...): whitespace-separated numbers of a file."""
    with open(fname) as r:
        return [float(t) for t in r.read().split()]
