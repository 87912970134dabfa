"""Host containers mirroring the reference's return types.

SpectralArray mirrors src/spectralarray.jl:5-16 (a 0-based OffsetArray
wrapper whose axes are l ranges); BlockSpectralMatrix mirrors
src/blockspectralmatrix.jl:5-25 (a dense matrix built by hvcat of
SpectralArrays, remembering the l ranges of its block rows and columns).
`parent` is the dense column-major numpy array the C ABI writes into.
"""
import numpy as np


class SpectralArray:
    def __init__(self, parent, axes=None):
        parent = np.asarray(parent)
        if axes is None:
            axes = tuple(range(0, n) for n in parent.shape)
        axes = tuple(a if isinstance(a, range) else range(a[0], a[1] + 1) for a in axes)
        if tuple(len(a) for a in axes) != parent.shape:
            raise ValueError("axes %r do not match shape %r" % (axes, parent.shape))
        self.parent = parent
        self.axes = axes

    @property
    def shape(self):
        return self.parent.shape

    def _idx(self, key):
        if not isinstance(key, tuple):
            key = (key,)
        out = []
        for k, ax in zip(key, self.axes):
            if isinstance(k, slice):
                start = ax.start if k.start is None else k.start
                stop = ax.stop if k.stop is None else k.stop + 1  # l ranges are inclusive, like Julia
                out.append(slice(start - ax.start, stop - ax.start, k.step))
            else:
                if k not in ax:
                    raise IndexError("l = %d outside axis %r" % (k, ax))
                out.append(k - ax.start)
        return tuple(out)

    def __getitem__(self, key):
        return self.parent[self._idx(key)]

    def __setitem__(self, key, value):
        self.parent[self._idx(key)] = value

    def __neg__(self):
        return SpectralArray(-self.parent, self.axes)

    def __array__(self, dtype=None, copy=None):
        return self.parent if dtype is None else self.parent.astype(dtype)

    def __repr__(self):
        return "SpectralArray(axes=%r, parent=%r)" % (self.axes, self.parent)


def SpectralVector(v, start=0):
    v = np.asarray(v, dtype=np.float64)
    return SpectralArray(v, (range(start, start + len(v)),))


def spectralzeros(*ranges):
    """Column-major zeros with the given l ranges (src/spectralarray.jl:79-80)."""
    ranges = tuple(r if isinstance(r, range) else range(r[0], r[1] + 1) for r in ranges)
    return SpectralArray(np.zeros(tuple(len(r) for r in ranges), dtype=np.float64, order="F"), ranges)


def spectralones(*ranges):
    ranges = tuple(r if isinstance(r, range) else range(r[0], r[1] + 1) for r in ranges)
    return SpectralArray(np.ones(tuple(len(r) for r in ranges), dtype=np.float64, order="F"), ranges)


class BlockSpectralMatrix:
    """Dense block matrix with per-block l ranges (src/blockspectralmatrix.jl:5-25)."""

    def __init__(self, parent, m_ells, n_ells):
        self.parent = parent
        self.m_ells = tuple(m_ells)
        self.n_ells = tuple(n_ells)

    @classmethod
    def hvcat(cls, rows):
        """rows: list of lists of SpectralArray, like Julia's [A B; C D]."""
        parent = np.asfortranarray(np.block([[np.asarray(b.parent) for b in row] for row in rows]))
        m_ells = tuple(row[0].axes[0] for row in rows)
        n_ells = tuple(b.axes[1] for b in rows[0])
        return cls(parent, m_ells, n_ells)

    def getblock(self, i, j):
        """Block (i, j), 0-based, as a SpectralArray with its l axes."""
        r0 = sum(len(r) for r in self.m_ells[:i])
        c0 = sum(len(c) for c in self.n_ells[:j])
        mi, nj = self.m_ells[i], self.n_ells[j]
        return SpectralArray(self.parent[r0:r0 + len(mi), c0:c0 + len(nj)], (mi, nj))

    @property
    def shape(self):
        return self.parent.shape

    def __array__(self, dtype=None, copy=None):
        return self.parent if dtype is None else self.parent.astype(dtype)
