"""Structured output container with Spitfire's ``Library``/``Dimension`` interface (spitfire/chemistry/library.py).

A ``Library`` is an N-dimensional table over named ``Dimension`` grids; properties are arrays shaped like the
grid. It is the output format of the reactor and SLFM front ends; ``save_to_file``/``load_from_file`` use pickle
(library.py:180-256) with plain-data state so files do not depend on this package's class layout.
"""

import pickle

import numpy as np


class Dimension:
    def __init__(self, name: str, values, log_scaled=False):
        values = np.array(values, dtype=np.float64)
        if not name.isidentifier():
            raise ValueError(f'Dimension name "{name}" must be a valid Python identifier')
        if values.ndim != 1:
            raise ValueError(f'Dimension "{name}": values must be one-dimensional')
        if values.size != np.unique(values).size:
            raise ValueError(f'Dimension "{name}": duplicate values')
        self._name = name
        self._values = values
        self._log_scaled = log_scaled

    def __repr__(self):
        return f'Dimension "{self._name}" spanning [{self.min}, {self.max}] with {self.npts} points'

    @property
    def name(self):
        return self._name

    @property
    def values(self):
        return self._values

    @property
    def min(self):
        return float(np.min(self._values))

    @property
    def max(self):
        return float(np.max(self._values))

    @property
    def npts(self):
        return self._values.size

    @property
    def log_scaled(self):
        return self._log_scaled


class LibraryIndexError(IndexError):
    pass


class Library:
    def __init__(self, *dimensions):
        self._dims = {d.name: d for d in dimensions}
        self._order = [d.name for d in dimensions]
        self._props = {}
        self._extra = {}
        for d in dimensions:
            setattr(self, d.name + '_name', d.name)
            setattr(self, d.name + '_values', d.values)
        shape = tuple(d.npts for d in dimensions)
        self._shape = shape
        grids = np.meshgrid(*[d.values for d in dimensions], indexing='ij') if dimensions else []
        for d, g in zip(dimensions, grids):
            setattr(self, d.name + '_grid', g)

    @property
    def extra_attributes(self):
        return self._extra

    def __setitem__(self, name, values):
        values = np.asarray(values, dtype=np.float64)
        if values.shape != self._shape:
            if values.size == int(np.prod(self._shape)):
                values = values.reshape(self._shape)
            else:
                raise LibraryIndexError(f'property "{name}" has shape {values.shape}, library shape {self._shape}')
        self._props[name] = values

    def __getitem__(self, name):
        if isinstance(name, str):
            return self._props[name]
        raise LibraryIndexError('index a Library by property name')

    def __contains__(self, name):
        return name in self._props

    @property
    def props(self):
        return list(self._props)

    @property
    def dims(self):
        return [self._dims[n] for n in self._order]

    @property
    def dim_names(self):
        return list(self._order)

    def dim(self, name):
        return self._dims[name]

    @property
    def shape(self):
        return self._shape

    @property
    def size(self):
        return int(np.prod(self._shape))

    def get_empty_dataset(self):
        return np.zeros(self._shape)

    def remove(self, *names):
        for n in names:
            self._props.pop(n)

    def __getstate__(self):
        return dict(dimensions={n: dict(name=n, values=self._dims[n].values, log_scaled=self._dims[n].log_scaled)
                                for n in self._order},
                    dim_ordering={i: n for i, n in enumerate(self._order)}, properties=dict(self._props),
                    extra_attributes=dict(self._extra))

    def __setstate__(self, st):
        order = [st['dim_ordering'][i] for i in range(len(st['dim_ordering']))]
        dims = [Dimension(st['dimensions'][n]['name'], st['dimensions'][n]['values'],
                          st['dimensions'][n].get('log_scaled', False)) for n in order]
        self.__init__(*dims)
        for k, v in st['properties'].items():
            self[k] = v
        self._extra = dict(st.get('extra_attributes', {}))

    def save_to_file(self, file_name):
        with open(file_name, 'wb') as f:
            pickle.dump(self.__getstate__(), f)

    @classmethod
    def load_from_file(cls, file_name):
        with open(file_name, 'rb') as f:
            st = pickle.load(f)
        lib = cls.__new__(cls)
        lib.__setstate__(st)
        return lib
