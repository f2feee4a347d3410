"""Structured output container with Spitfire's ``Library``/``Dimension`` interface (spitfire/chemistry/library.py).

A ``Library`` is an N-dimensional table over named ``Dimension`` grids; properties are arrays shaped like the
grid. It is the output format of the reactor and flamelet front ends and of the library builders. The interface
follows library.py:21-452:
* per dimension `x`, the attributes `x_name`, `x_values`, `x_min`, `x_max`, `x_npts`, `x_log_scaled` and `x_grid`
  (the N-dimensional meshgrid);
* `lib['prop']` for a property; `lib[s0, s1, ...]` (one slice or integer per dimension) for a new, sliced library
  that keeps every dimension (`lib[:]` is the whole library);
* `Library.copy` / `deepcopy` / `squeeze` / `swapaxes`, `scale_dimension` / `remap_dimension`;
* `save_to_file` / `load_from_file` (pickle of plain data, so files do not depend on this package's class layout)
  and `save_to_text_directory`.

`save_to_text_directory` replaces an existing directory only with overwrite=True: the reference asks on standard
input first, which a library called from batch jobs should not do.
"""

import copy as _copy
import os
import pickle
import shutil

import numpy as np


class _ReferenceUnpickler(pickle.Unpickler):
    """Unpickler that reads files written by the reference package: spitfire.chemistry.library.{Library, Dimension}
    and spitfire.chemistry.mechanism.ChemicalMechanismSpec become this package's classes, and numpy's pre-2.0
    module path numpy.core is read as numpy._core where that exists."""

    _MAP = {('spitfire.chemistry.library', 'Library'): ('spitfire_gb300.library', 'Library'),
            ('spitfire.chemistry.library', 'Dimension'): ('spitfire_gb300.library', 'Dimension'),
            ('spitfire.chemistry.library', 'LibraryIndexError'): ('spitfire_gb300.library', 'LibraryIndexError'),
            ('spitfire.chemistry.mechanism', 'ChemicalMechanismSpec'): ('spitfire_gb300.mechanism',
                                                                       'ChemicalMechanismSpec')}

    def find_class(self, module, name):
        module, name = self._MAP.get((module, name), (module, name))
        if module.startswith('numpy.core') and hasattr(np, '_core'):
            module = 'numpy._core' + module[len('numpy.core'):]
        return super().find_class(module, name)


class Dimension:
    """A named, one-dimensional grid of unique values (library.py:21-89)."""

    def __init__(self, name: str, values, log_scaled=False):
        values = np.array(values, dtype=np.float64)
        if not name.isidentifier():
            raise ValueError(f'Dimension name "{name}" must be a valid Python identifier (no hyphens or spaces)')
        if values.ndim != 1:
            raise ValueError(f'Dimension "{name}": values must be one-dimensional (ravel() them)')
        if values.size != np.unique(values).size:
            raise ValueError(f'Dimension "{name}": duplicate values')
        self._name = name
        self._values = values
        self._log_scaled = log_scaled

    def __str__(self):
        return f'Dimension "{self._name}" spanning [{self.min}, {self.max}] with {self.npts} points'

    def __repr__(self):
        return f'Dimension(name="{self._name}", min={self.min}, max={self.max}, npts={self.npts})'

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


def _as_dimension(d):
    if isinstance(d, Dimension):
        return Dimension(d.name, d.values, d.log_scaled)
    return Dimension(d[0], d[1], False if len(d) == 2 else d[2])


class Library:
    """An N-dimensional table of properties over Dimension grids; see the module docstring."""

    def __init__(self, *dimensions):
        dims = [_as_dimension(d) for d in dimensions]
        self._dims = {d.name: d for d in dims}
        self._order = [d.name for d in dims]
        self._props = {}
        self._extra = {}
        self._set_grid()

    def _set_grid(self):
        dims = self.dims
        self._shape = tuple(d.npts for d in dims)
        grids = np.meshgrid(*[d.values for d in dims], indexing='ij') if dims else []
        for d, g in zip(dims, grids):
            setattr(self, d.name, d.name)
            for attr in ('name', 'values', 'min', 'max', 'npts', 'log_scaled'):
                setattr(self, d.name + '_' + attr, getattr(d, attr))
            setattr(self, d.name + '_grid', g.copy())

    # ------------------------------------------------------------------------------------------ dimensions
    def scale_dimension(self, dim_name, multiplier):
        """Multiply a dimension's values by `multiplier` (library.py:140-144)."""
        self.remap_dimension(dim_name, lambda x: multiplier * x)

    def remap_dimension(self, dim_name, mapping):
        """Replace a dimension's values by mapping(values) (library.py:146-151); the dimension is no longer marked
        log-scaled, as in the reference."""
        if dim_name not in self._dims:
            raise KeyError(f'Invalid dimension name "{dim_name}" for this library')
        self._dims[dim_name] = Dimension(dim_name, mapping(self._dims[dim_name].values))
        self._set_grid()

    @property
    def extra_attributes(self):
        return self._extra

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

    # ------------------------------------------------------------------------------------------ properties
    def __setitem__(self, name, values):
        """lib['prop'] = array shaped like the grid (an array of the grid's size is reshaped), or a number that
        fills the grid (library.py:330-347)."""
        if isinstance(values, (float, int)) and not isinstance(values, bool):
            if name not in self._props:
                self._props[name] = self.get_empty_dataset()
            self._props[name].fill(float(values))
            return
        if not isinstance(values, (np.ndarray, list, tuple)):
            raise TypeError(f'Library["{name}"] = values needs an array or a number, received {type(values)}')
        values = np.asarray(values, dtype=np.float64)
        if values.shape != self._shape:
            if values.size != self.size:
                raise ValueError(f'property "{name}" has shape {values.shape}, the library grid {self._shape}')
            values = values.reshape(self._shape)
        self._props[name] = values

    def __getitem__(self, key):
        """lib['prop'] for a property; lib[s0, s1, ...] with one slice or integer per dimension (lib[:] for all of
        them) for a new library over the sliced grid that keeps every dimension, its properties views of this
        library's (library.py:349-389)."""
        if isinstance(key, str):
            return self._props[key]
        if isinstance(key, slice):
            key = (key,) * len(self._order) if key == slice(None) else (key,)
        if not isinstance(key, tuple):
            raise LibraryIndexError(f'Library[...] takes one property name or standard slices, received {key!r}')
        if len(key) != len(self._order):
            raise LibraryIndexError(f'Library[...] slicing needs one argument per dimension ({len(self._order)}), '
                                    f'received {len(key)}')
        for k in key:
            if isinstance(k, bool) or not isinstance(k, (slice, int, np.integer)):
                raise LibraryIndexError(f'Library[...] takes one property name or standard slices, received {key!r}')
        new_dims = []
        for d, k in zip(self.dims, key):
            v = d.values[k]
            new_dims.append(Dimension(d.name, np.atleast_1d(v), d.log_scaled))
        out = Library(*new_dims)
        for p, v in self._props.items():
            out._props[p] = v[key].reshape(out.shape)
        out._extra = dict(self._extra)
        return out

    def __contains__(self, name):
        return name in self._props

    @property
    def props(self):
        return list(self._props)

    def get_empty_dataset(self):
        return np.zeros(self._shape)

    def add_empty_property(self, name):
        self._props[name] = self.get_empty_dataset()

    def remove(self, *names):
        for n in names:
            self._props.pop(n)

    # ------------------------------------------------------------------------------------------ copies
    def __copy__(self):
        out = Library(*self.dims)
        out._props = dict(self._props)
        out._extra = dict(self._extra)
        return out

    def __deepcopy__(self, memo=None):
        out = Library(*[Dimension(d.name, d.values.copy(), d.log_scaled) for d in self.dims])
        out._props = {p: v.copy() for p, v in self._props.items()}
        out._extra = dict(self._extra)
        return out

    @classmethod
    def copy(cls, library):
        """A new library sharing the property arrays (library.py:283-286)."""
        return _copy.copy(library)

    @classmethod
    def deepcopy(cls, library):
        """A new library with copies of everything (library.py:288-291)."""
        return _copy.deepcopy(library)

    @classmethod
    def squeeze(cls, library):
        """The library without its single-value dimensions (library.py:293-315); with none left, the dictionary
        {'properties': {...}, 'dimensions': {name: (value, log_scaled)}, 'extra_attributes': {...}}."""
        keep = [d for d in library.dims if d.npts > 1]
        if not keep:
            return dict(properties={p: np.squeeze(library[p]) for p in library.props},
                        dimensions={d.name: (np.squeeze(d.values), d.log_scaled) for d in library.dims},
                        extra_attributes=library.extra_attributes)
        out = Library(*keep)
        for p in library.props:
            out[p] = np.squeeze(library[p])
        out._extra = dict(library.extra_attributes)
        return out

    @classmethod
    def swapaxes(cls, library, idx1, idx2):
        """The library with dimensions idx1 and idx2 exchanged (library.py:317-328)."""
        names = library.dim_names
        if len(names) < 2:
            raise ValueError('Cannot swap dimensions of a library with one dimension.')
        names[idx1], names[idx2] = names[idx2], names[idx1]
        out = Library(*[Dimension(n, library.dim(n).values, library.dim(n).log_scaled) for n in names])
        for p in library.props:
            out[p] = np.swapaxes(library[p], idx1, idx2)
        out._extra = dict(library.extra_attributes)
        return out

    # ------------------------------------------------------------------------------------------ text
    def __str__(self):
        lines = [f'Spitfire Library with {len(self._order)} dimensions and {len(self._props)} properties',
                 '-' * 42]
        lines += [f'{i + 1}. {d}' for i, d in enumerate(self.dims)]
        lines.append('-' * 42)
        lines += [f'{k:20}, min = {np.min(v)} max = {np.max(v)}' for k, v in self._props.items()]
        lines.append(f'Extra attributes: {self._extra}')
        return '\n' + '\n'.join(lines) + '\n'

    def __repr__(self):
        return (f'Library(ndim={len(self._order)}, nproperties={len(self._props)}): '
                f'{", ".join(repr(d) for d in self.dims)}; properties [{", ".join(self._props)}]')

    # ------------------------------------------------------------------------------------------ files
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
        """Load a library saved by save_to_file, or one the reference wrote: its save_to_file pickles the
        spitfire.chemistry.library.Library object itself (library.py:180-183), with the mechanism's
        ChemicalMechanismSpec among the extra attributes, and its version-1.0 files pickle the plain dictionary
        (library.py:246-256). Reference classes are mapped onto this package's Library, Dimension and
        ChemicalMechanismSpec, whose __setstate__ read the same dictionaries."""
        with open(file_name, 'rb') as f:
            st = _ReferenceUnpickler(f).load()
        if isinstance(st, Library):
            return st
        lib = cls.__new__(cls)
        lib.__setstate__(st)
        return lib

    def save_to_text_directory(self, output_directory, ravel_order='F', format='%.14e', overwrite=False):
        """Plain-text dump for other codes (library.py:185-244): metadata_independent_variables.txt (dimension
        names), metadata_dependent_variables.txt (property names, spaces as underscores),
        metadata_user_defined_attributes.txt, bulkdata_ivar_<dim>.txt and bulkdata_dvar_<prop>.txt (flattened in
        ravel_order, 'F' by default)."""
        if os.path.isdir(output_directory):
            if not overwrite:
                raise FileExistsError(f'{output_directory} exists; pass overwrite=True to replace it')
            shutil.rmtree(output_directory)
        os.mkdir(output_directory)
        under = {p: p.replace(' ', '_') for p in self._props}
        with open(os.path.join(output_directory, 'metadata_independent_variables.txt'), 'w') as f:
            for d in self.dims:
                f.write(d.name + '\n')
        with open(os.path.join(output_directory, 'metadata_dependent_variables.txt'), 'w') as f:
            for p in self._props:
                f.write(under[p] + '\n')
        with open(os.path.join(output_directory, 'metadata_user_defined_attributes.txt'), 'w') as f:
            f.write(str(self._extra))
        for d in self.dims:
            np.savetxt(os.path.join(output_directory, f'bulkdata_ivar_{d.name}.txt'), d.values, fmt=format)
        for p, v in self._props.items():
            np.savetxt(os.path.join(output_directory, f'bulkdata_dvar_{under[p]}.txt'), v.ravel(order=ravel_order),
                       fmt=format)
