"""Minimal stand-in for the few pandas calls the reference makes on its MC path.

Test infrastructure only: it lets the mounted reference (chromo) import and run
in a container without pandas.  It covers ``DataFrame(columns=...)``,
``append(dict, ignore_index=True)``, ``len``, ``.loc/.at[i, col]`` get/set,
``.iloc[i].attr`` and ``to_dict(orient='records')`` -- the calls made by
``chromo/binders.pyx:210-238`` and ``chromo/fields.pyx:503,528,687-712`` --
and ``copy()``, ``df[col] *= x`` / ``/= x``, ``df[col][i]`` and ``df.index``,
made by ``chromo/util/rediscretize.py:364-398,958-991``.  As in pandas, a copy
has its own rows, while objects held in cells (the cross-talk dicts) are
shared.
"""


class _Row:
    def __init__(self, d):
        object.__setattr__(self, "_d", d)

    def __getattr__(self, k):
        try:
            return self._d[k]
        except KeyError as e:
            raise AttributeError(k) from e

    def __getitem__(self, k):
        return self._d[k]

    def to_dict(self):
        return dict(self._d)


class _Indexer:
    def __init__(self, df):
        self._df = df

    def __getitem__(self, key):
        i, col = key
        return self._df._rows[i][col]

    def __setitem__(self, key, value):
        i, col = key
        self._df._rows[i][col] = value


class _ILoc:
    def __init__(self, df):
        self._df = df

    def __getitem__(self, i):
        return _Row(self._df._rows[i])


class _Column:
    def __init__(self, df, col):
        self._df, self._col = df, col

    def __getitem__(self, i):
        return self._df._rows[i][self._col]

    def __imul__(self, x):
        for r in self._df._rows:
            r[self._col] = r[self._col] * x
        return self

    def __itruediv__(self, x):
        for r in self._df._rows:
            r[self._col] = r[self._col] / x
        return self


class DataFrame:
    def __init__(self, data=None, columns=None, **kwargs):
        self._rows = []
        self.columns = list(columns) if columns is not None else []
        if isinstance(data, list):
            for d in data:
                self._rows.append(dict(d))

    def append(self, d, ignore_index=True):
        out = DataFrame(columns=self.columns)
        out._rows = [dict(r) for r in self._rows] + [dict(d)]
        return out

    def __len__(self):
        return len(self._rows)

    @property
    def loc(self):
        return _Indexer(self)

    @property
    def at(self):
        return _Indexer(self)

    @property
    def iloc(self):
        return _ILoc(self)

    def to_dict(self, orient="records"):
        return [dict(r) for r in self._rows]

    def equals(self, other):
        return self._rows == other._rows

    def copy(self, deep=True):
        out = DataFrame(columns=self.columns)
        out._rows = [dict(r) for r in self._rows]
        return out

    @property
    def index(self):
        return range(len(self._rows))

    def __getitem__(self, col):
        return _Column(self, col)

    def __setitem__(self, col, value):
        if isinstance(value, _Column):
            return  # the in-place column arithmetic above already updated the rows
        for r in self._rows:
            r[col] = value


class MultiIndex:
    @staticmethod
    def from_product(*a, **k):
        return None


def read_csv(*a, **k):
    raise NotImplementedError("pandas stand-in: read_csv is not available")
