"""Multi-indices, limiters and adaptive multi-index sets: the reference's
MultiIndex (src/MultiIndices/MultiIndex.cpp), MultiIndexLimiter
(MParT/MultiIndices/MultiIndexLimiter.h, src/MultiIndices/MultiIndexLimiter.cpp)
and MultiIndexSet (src/MultiIndices/MultiIndexSet.cpp, with the default
neighbourhood of src/MultiIndices/MultiIndexNeighborhood.cpp), with the names
of its Python binding (bindings/python/src/MultiIndex.cpp:60-240).  Host-side
set algebra used to build the sets that define map components; fix() gives
the FixedMultiIndexSet that CreateComponent takes.

The set keeps the reference's bookkeeping, which decides the order of every
query: each multi-index it has seen has a global number in order of first
appearance; activating one adds its forward and backward neighbours that the
limiter allows as inactive entries, and edges between existing entries are
kept as ordered sets of global numbers per entry and direction."""
from __future__ import annotations

import copy as _copy
import math

import numpy as np


class MultiIndex:
    """MultiIndex(), MultiIndex(length), MultiIndex(length, value) or
    MultiIndex(sequence of orders)."""

    def __init__(self, *args):
        if not args:
            v = ()
        elif len(args) == 1 and not isinstance(args[0], (int, np.integer)):
            v = tuple(int(x) for x in np.asarray(args[0]).reshape(-1))
            if any(x < 0 for x in v):
                raise ValueError("MultiIndex: orders must be non-negative")
        else:
            length = int(args[0])
            val = int(args[1]) if len(args) > 1 else 0
            v = (val,) * length
        self._v = list(v)

    # -- the reference's accessors --------------------------------------------
    def tolist(self):
        return list(self._v)

    Vector = tolist

    def sum(self):
        return sum(self._v)

    def max(self):
        return max(self._v) if self._v else 0

    def count_nonzero(self):
        return sum(1 for x in self._v if x)

    def HasNonzeroEnd(self):
        """The last entry is nonzero (MultiIndex::HasNonzeroEnd)."""
        return bool(self._v) and self._v[-1] != 0

    def __len__(self):
        return len(self._v)

    def __getitem__(self, i):
        # MultiIndex::Get: an index past the end reads 0, beyond it throws.
        i = int(i)
        if i < 0 or i > len(self._v):
            raise IndexError(f"Tried to access index {i} of a multiindex with only {len(self._v)} components.")
        return self._v[i] if i < len(self._v) else 0

    def __setitem__(self, i, val):
        i = int(i)
        if i < 0 or i >= len(self._v):
            raise IndexError(f"Tried to set the value of index {i} on an multiindex with only {len(self._v)} "
                             "components.")
        self._v[i] = int(val)

    def __iter__(self):
        return iter(list(self._v))

    def __str__(self):
        return " ".join(str(x) for x in self._v)

    __repr__ = __str__

    def _key(self):
        return tuple(self._v)

    def __hash__(self):
        return hash(self._key())

    # Ordering of MultiIndex::operator<: length, total order, maximum, then
    # entry by entry.
    def _rank(self):
        return (len(self._v), sum(self._v), self.max(), tuple(self._v))

    def __eq__(self, other):
        return isinstance(other, MultiIndex) and self._v == other._v

    def __ne__(self, other):
        return not self == other

    __neq__ = __ne__

    def __lt__(self, other):
        return self._rank() < other._rank()

    def __gt__(self, other):
        return other._rank() < self._rank()

    def __le__(self, other):
        return not self > other

    def __ge__(self, other):
        return not self < other


def _multi(m) -> MultiIndex:
    return m if isinstance(m, MultiIndex) else MultiIndex(m)


# ---- limiters (MultiIndexLimiter) -------------------------------------------
class TotalOrder:
    """Terms of total order at most maxOrder."""

    def __init__(self, totalOrder):
        self.totalOrder = int(totalOrder)

    def __call__(self, multi):
        return _multi(multi).sum() <= self.totalOrder


class Dimension:
    """Terms whose nonzero entries all lie in [lowerDim, lowerDim + length)."""

    def __init__(self, lowerDim, length):
        self.lowerDim, self.length = int(lowerDim), int(length)

    def __call__(self, multi):
        m = _multi(multi)
        return all(m[i] == 0 for i in range(self.lowerDim)) and \
            all(m[i] == 0 for i in range(self.lowerDim + self.length, len(m)))


class Anisotropic:
    """Terms with prod_i weights[i]^multi[i] >= epsilon."""

    def __init__(self, weights, epsilon):
        self.weights = [float(w) for w in weights]
        self.epsilon = float(epsilon)
        for w in self.weights:
            if w > 1.0 or w < 0.0:
                raise ValueError(f"AnisotropicLimiter requires all weights have to be in [0,1]. Got weight {w:f}")
        if self.epsilon >= 1.0 or self.epsilon <= 0.0:
            raise ValueError(f"AnisotropicLimiter requires epsilon to be in (0,1). Got epsilon = {self.epsilon:f}")

    def __call__(self, multi):
        v = _multi(multi)._v
        if len(v) != len(self.weights):
            return False
        prod = 1.0
        for w, k in zip(self.weights, v):
            prod *= math.pow(w, k)
        return prod >= self.epsilon


class MaxDegree:
    """MaxDegree(maxDegree, length) or MaxDegree(sequence of per-dimension maxima)."""

    def __init__(self, maxDegree, length=None):
        self.maxDegrees = [int(maxDegree)] * int(length) if length is not None else [int(d) for d in maxDegree]

    def __call__(self, multi):
        v = _multi(multi)._v
        return len(v) == len(self.maxDegrees) and all(a <= b for a, b in zip(v, self.maxDegrees))


class NoneLim:
    """Every multi-index."""

    def __call__(self, multi):
        return True


class Separable:
    """No cross terms with the last input: the last entry is zero or the whole order."""

    def __call__(self, multi):
        m = _multi(multi)
        return not m.HasNonzeroEnd() or m.sum() == m[len(m) - 1]


class NonzeroDiag:
    """Terms whose last entry is nonzero."""

    def __call__(self, multi):
        return _multi(multi).HasNonzeroEnd()


class And:
    def __init__(self, a, b):
        self.a, self.b = a, b

    def __call__(self, multi):
        return bool(self.a(multi)) and bool(self.b(multi))


class Or:
    def __init__(self, a, b):
        self.a, self.b = a, b

    def __call__(self, multi):
        return bool(self.a(multi)) or bool(self.b(multi))


class Xor:
    def __init__(self, a, b):
        self.a, self.b = a, b

    def __call__(self, multi):
        return bool(self.a(multi)) != bool(self.b(multi))


# ---- MultiIndexSet ----------------------------------------------------------
class MultiIndexSet:
    """MultiIndexSet(length[, limiter]), MultiIndexSet(2-D array or list of
    terms: one row per term, added in order) or MultiIndexSet(length, terms)."""

    def __init__(self, *args):
        if not args or len(args) > 2:
            raise TypeError("MultiIndexSet(length[, limiter]), MultiIndexSet(length, terms) or MultiIndexSet(multis)")
        terms = ()
        if isinstance(args[0], (int, np.integer)):
            length, limiter = int(args[0]), NoneLim()
            if len(args) > 1:
                if callable(args[1]):
                    limiter = args[1]
                else:
                    terms = args[1]
        else:
            arr = np.asarray(args[0])
            if arr.ndim != 2:
                raise ValueError("Expected array with ndims = 2")
            length, limiter, terms = arr.shape[1], NoneLim(), arr
        self._length = length
        self._limiter = limiter
        self._all = []          # every entry, by global number (tuples)
        self._global = {}       # tuple -> global number
        self._g2a = []          # global number -> active index or -1
        self._a2g = []          # active index -> global number
        self._in = []           # backward edges (sets of global numbers)
        self._out = []          # forward edges
        self._maxOrders = [0] * length
        for t in terms:
            self.AddActive(t)

    # -- construction (MultiIndexSet::CreateTotalOrder / CreateTensorProduct) --
    @staticmethod
    def CreateTotalOrder(length, maxOrder, limiter=None):
        if int(length) <= 0:
            raise ValueError("MultiIndexSet::CreateTotalOrder: length must be positive")
        limiter = limiter or NoneLim()
        out = MultiIndexSet(int(length), limiter)
        base = [0] * int(length)

        def fill(dim):
            cur = sum(base[:dim])
            for i in range(int(maxOrder) - cur + 1):
                if dim == len(base) - 1:
                    base[-1] = i
                    if limiter(MultiIndex(base)):
                        out.AddActive(base)
                else:
                    for k in range(dim + 1, len(base)):
                        base[k] = 0
                    base[dim] = i
                    fill(dim + 1)

        fill(0)
        return out

    @staticmethod
    def CreateTensorProduct(length, maxOrder, limiter=None):
        if int(length) <= 0:
            raise ValueError("MultiIndexSet::CreateTensorProduct: length must be positive")
        limiter = limiter or NoneLim()
        out = MultiIndexSet(int(length), limiter)
        base = [0] * int(length)

        def fill(dim):
            for i in range(int(maxOrder) + 1):
                if dim == len(base) - 1:
                    base[-1] = i
                    if limiter(MultiIndex(base)):
                        out.AddActive(base)
                else:
                    for k in range(dim + 1, len(base)):
                        base[k] = 0
                    base[dim] = i
                    fill(dim + 1)

        fill(0)
        return out

    @staticmethod
    def CreateSeparableTotalOrder(length, maxOrder):
        return MultiIndexSet.CreateTotalOrder(length, maxOrder, Separable())

    @staticmethod
    def CreateNonzeroDiagTotalOrder(length, maxOrder):
        return MultiIndexSet.CreateTotalOrder(length, maxOrder, NonzeroDiag())

    # -- size and access -------------------------------------------------------
    def Size(self):
        return len(self._a2g)

    def Length(self):
        return self._length

    def __len__(self):
        return self._length

    def IndexToMulti(self, activeIndex):
        return MultiIndex(self._all[self._a2g[int(activeIndex)]])

    def at(self, activeIndex):
        i = int(activeIndex)
        if i < 0 or i >= len(self._a2g):
            raise IndexError(f"active index {i} out of range for a set of {len(self._a2g)} terms")
        return self.IndexToMulti(i)

    __getitem__ = at

    def MultiToIndex(self, multi):
        g = self._global.get(_multi(multi)._key())
        return -1 if g is None else self._g2a[g]

    def MaxOrders(self):
        return list(self._maxOrders)

    def NonzeroDiagonalEntries(self):
        return [i for i, g in enumerate(self._a2g) if self._all[g] and self._all[g][-1] != 0]

    def GetLimiter(self):
        return self._limiter

    @property
    def _terms(self):
        return [self._all[g] for g in self._a2g]

    def Multis(self):
        return [np.array(t, dtype=np.uint32) for t in self._terms]

    def _dense(self):
        return np.ascontiguousarray(np.array(self._terms, dtype=np.uint32).reshape(self.Size(), self._length))

    def fix(self, compress=True):
        """The active terms, in order, as a FixedMultiIndexSet (MultiIndexSet::Fix)."""
        from . import FixedMultiIndexSet
        if not self.Size():
            return FixedMultiIndexSet(self._length, nzStarts=[0])
        return FixedMultiIndexSet.from_multis(self._dense())

    Fix = fix

    def DeepCopy(self):
        return _copy.deepcopy(self)

    # -- bookkeeping (MultiIndexSet.cpp:239-430, 690-711) ------------------------
    def _lim(self, key):
        return bool(self._limiter(MultiIndex(key)))

    def _add_multi(self, key):
        self._all.append(key)
        g = len(self._all) - 1
        self._global[key] = g
        self._g2a.append(-1)
        self._in.append(set())
        self._out.append(set())
        self._add_forward(g, False)
        self._add_backward(g, False)
        return g

    def _add_inactive(self, key):
        g = self._global.get(key)
        if g is not None:
            return g
        if self._lim(key):
            return self._add_multi(key)
        return -1

    def _add_forward(self, g, add_inactive):
        v = self._all[g]
        for d in range(self._length):
            f = v[:d] + (v[d] + 1,) + v[d + 1:]
            if self._lim(f):
                h = self._global.get(f)
                if h is not None:
                    self._in[h].add(g)
                    self._out[g].add(h)
                elif add_inactive:
                    self._add_inactive(f)

    def _add_backward(self, g, add_inactive):
        v = self._all[g]
        for d in range(self._length):
            if v[d] == 0:
                continue
            b = v[:d] + (v[d] - 1,) + v[d + 1:]
            if self._lim(b):
                h = self._global.get(b)
                if h is not None:
                    self._out[h].add(g)
                    self._in[g].add(h)
                elif add_inactive:
                    self._add_inactive(b)

    def _activate(self, g):
        if self._g2a[g] >= 0:
            return
        self._a2g.append(g)
        self._g2a[g] = len(self._a2g) - 1
        for d, k in enumerate(self._all[g]):
            if k:
                self._maxOrders[d] = max(self._maxOrders[d], k)
        self._add_forward(g, True)
        self._add_backward(g, True)

    def _active(self, g):
        return self._g2a[g] >= 0

    def _admissible(self, g):
        key = self._all[g]
        if not self._lim(key):
            return False
        if self._active(g):
            return True
        return sum(1 for h in self._in[g] if self._active(h)) == sum(1 for k in key if k)

    def _key(self, multi):
        key = _multi(multi)._key()
        if len(key) != self._length:
            raise ValueError(f"multi-index of length {len(key)} in a set of length {self._length}")
        return key

    # -- the reference's methods ----------------------------------------------
    def AddActive(self, multi):
        """Adds the term (if the limiter allows it) and activates it; its active
        index, or -1."""
        g = self._add_inactive(self._key(multi))
        if g < 0:
            return -1
        self._activate(g)
        return self._g2a[g]

    def append(self, multi):
        self.AddActive(multi)
        return self

    def __iadd__(self, other):
        if isinstance(other, MultiIndexSet):
            self.union(other)
        else:
            self.AddActive(other)
        return self

    def Activate(self, multi):
        g = self._global.get(self._key(multi))
        if g is None or not self._admissible(g):
            raise ValueError("MultiIndexSet::Activate: the multi-index is not an admissible member of the set")
        self._activate(g)

    def IsActive(self, multi):
        g = self._global.get(self._key(multi))
        return g is not None and self._active(g)

    def IsAdmissible(self, multi):
        g = self._global.get(self._key(multi))
        return g is not None and self._admissible(g)

    def IsExpandable(self, activeIndex):
        g = self._a2g[int(activeIndex)]
        return any(not self._active(h) and self._admissible(h) for h in sorted(self._out[g]))

    def NumActiveForward(self, activeIndex):
        return sum(1 for h in self._out[self._a2g[int(activeIndex)]] if self._active(h))

    def NumForward(self, activeIndex):
        return len(self._out[self._a2g[int(activeIndex)]])

    def Frontier(self):
        return [a for a in range(self.Size()) if self.IsExpandable(a)]

    def StrictFrontier(self):
        return [a for a in self.Frontier() if not any(self._active(h) for h in self._out[self._a2g[a]])]

    def Margin(self):
        return [MultiIndex(self._all[g]) for g in range(len(self._all))
                if not self._active(g) and any(self._active(h) for h in self._in[g])]

    def ReducedMargin(self):
        """Inactive entries whose backward neighbours in the set are all active,
        by global number."""
        return [MultiIndex(self._all[g]) for g in range(len(self._all))
                if not self._active(g) and all(self._active(h) for h in self._in[g])]

    def ReducedMarginDim(self, dim):
        dim = int(dim)
        out = []
        for g in range(len(self._all)):
            if self._active(g):
                continue
            ins = self._in[g]
            if all(self._active(h) for h in ins) and any(self._all[h][dim] < self._all[g][dim] for h in ins):
                out.append(MultiIndex(self._all[g]))
        return out

    def Expand(self, activeIndex=None):
        """Expand(activeIndex): activates that term's admissible forward
        neighbours.  Expand(): those of every frontier term, collected before
        any is activated (a term reached from several frontier terms is
        returned once for each).  Returns the new active indices."""
        if activeIndex is not None:
            a = int(activeIndex)
            if a < 0 or a >= self.Size():
                raise IndexError(f"Invalid index passed to MultiIndexSet::Expand.  A value of {a} was passed to the "
                                 f"function, but only {self.Size()} active components exist in the set.")
            new = []
            for h in sorted(self._out[self._a2g[a]]):
                if self._admissible(h) and not self._active(h):
                    self._activate(h)
                    new.append(self._g2a[h])
            return new
        pending = []
        for a in self.Frontier():
            for h in sorted(self._out[self._a2g[a]]):
                if self._admissible(h) and not self._active(h):
                    pending.append(h)
        out = []
        for h in pending:
            self._activate(h)
            out.append(self._g2a[h])
        return out

    def union(self, rhs):
        """Adds rhs's entries the limiter allows, active ones active; returns
        how many terms became active."""
        old = self.Size()
        for g, key in enumerate(rhs._all):
            if self._lim(key):
                if rhs._g2a[g] < 0:
                    self._add_inactive(key)
                else:
                    self._activate(self._add_inactive(key))
        return self.Size() - old

    Union = union

    def SetLimiter(self, limiter):
        """Replaces the limiter: every active term must satisfy it; inactive
        entries that do not lose their edges."""
        self._limiter = limiter
        g = 0
        while g < len(self._all):
            key = self._all[g]
            if self._active(g):
                if not self._lim(key):
                    raise ValueError("Invalid limiter passed to MultiIndexSet::SetLimiter.  The active multi-index, "
                                     f"{list(key)}, is not valid with the new limiter.")
                self._add_forward(g, True)
            elif not self._lim(key):
                for h in self._in[g]:
                    self._out[h].discard(g)
                self._in[g].clear()
            g += 1
