"""The Library / Dimension output container (spitfire_gb300/library.py) against the behaviour of the reference's
spitfire/chemistry/library.py and its tests (tests/tabulation/test_library_*.py): dimension checks, grid
attributes, slicing, copies, squeeze and swapaxes, dimension remapping, pickle round trips and the text dump.
"""
import os

import numpy as np
import pytest

from spitfire_gb300.library import Dimension, Library, LibraryIndexError


def _lib2():
    l1 = Library(Dimension('x', np.linspace(0, 1, 4)), Dimension('y', np.linspace(-1, 1, 3)))
    l1['f'] = l1.x_grid + 10. * l1.y_grid
    l1['g'] = np.exp(l1.x_grid * l1.y_grid)
    l1.extra_attributes['name'] = 'two'
    return l1


@pytest.mark.parametrize('name,values', [('x-y', [0., 1.]), ('x y', [0., 1.]), ('x', [[0., 1.], [2., 3.]]),
                                         ('x', [0., 1., 1.])])
def test_dimension_rejects_bad_names_shapes_and_duplicates(name, values):
    with pytest.raises(ValueError):
        Dimension(name, np.array(values))


def test_grid_attributes():
    lib = _lib2()
    assert lib.shape == (4, 3) and lib.size == 12
    assert lib.x_name == 'x' and lib.x == 'x' and lib.y_npts == 3
    assert lib.x_min == 0. and lib.x_max == 1. and not lib.x_log_scaled
    np.testing.assert_array_equal(lib.x_values, np.linspace(0, 1, 4))
    gx, gy = np.meshgrid(np.linspace(0, 1, 4), np.linspace(-1, 1, 3), indexing='ij')
    np.testing.assert_array_equal(lib.x_grid, gx)
    np.testing.assert_array_equal(lib.y_grid, gy)
    assert lib.dim_names == ['x', 'y'] and lib.dim('y').npts == 3


def test_setitem_fill_reshape_and_errors():
    lib = _lib2()
    lib['c'] = 2.5
    assert np.all(lib['c'] == 2.5) and lib['c'].shape == lib.shape
    lib['flat'] = np.arange(12.)
    assert lib['flat'].shape == (4, 3)
    with pytest.raises(ValueError):
        lib['bad'] = np.arange(5.)
    with pytest.raises(TypeError):
        lib['bad'] = 'text'
    lib.add_empty_property('e')
    assert 'e' in lib and lib['e'].shape == lib.shape
    lib.remove('e', 'c')
    assert 'e' not in lib and 'c' not in lib


def test_slicing_one_dimension():
    l1 = Library(Dimension('x', np.linspace(0, 1, 16)))
    l1['f'] = l1.x_grid ** 2
    l2 = l1[:]
    np.testing.assert_array_equal(l2['f'], l1['f'])
    l3 = l1[3:9]
    np.testing.assert_array_equal(l3.x_grid, l1.x_grid[3:9])
    np.testing.assert_array_equal(l3['f'], l1['f'][3:9])
    assert l3.shape == (6,) and l3.size == 6
    l4 = l1[4:5]
    assert l4.shape == (1,)
    for bad in ((slice(None), slice(None)), ('f', slice(None)), (slice(None), 'g')):
        with pytest.raises(LibraryIndexError):
            l1[bad]


def test_slicing_two_dimensions_keeps_every_dimension():
    lib = _lib2()
    full = lib[:]
    assert full.shape == lib.shape
    np.testing.assert_array_equal(full['g'], lib['g'])
    part = lib[1:3, 0:2]
    assert part.shape == (2, 2)
    np.testing.assert_array_equal(part['f'], lib['f'][1:3, 0:2])
    np.testing.assert_array_equal(part.x_grid, lib.x_grid[1:3, 0:2])
    line = lib[:, 1]
    assert line.shape == (4, 1) and line.y_values[0] == 0.
    np.testing.assert_array_equal(line['f'][:, 0], lib['f'][:, 1])
    assert line.extra_attributes['name'] == 'two'
    with pytest.raises(LibraryIndexError):
        lib[1:2]


def test_squeeze():
    lib = _lib2()
    sq = Library.squeeze(lib[:, 1])
    assert sq.dim_names == ['x'] and sq.shape == (4,)
    np.testing.assert_array_equal(sq['f'], lib['f'][:, 1])
    point = Library.squeeze(lib[2, 1])
    assert isinstance(point, dict)
    assert point['properties']['f'] == lib['f'][2, 1]
    assert point['dimensions']['x'][0] == lib.x_values[2]


def test_copy_and_deepcopy():
    lib = _lib2()
    shallow = Library.copy(lib)
    deep = Library.deepcopy(lib)
    lib['f'][0, 0] = -123.
    assert shallow['f'][0, 0] == -123.
    assert deep['f'][0, 0] != -123.
    assert deep.extra_attributes['name'] == 'two'


def test_swapaxes():
    lib = _lib2()
    sw = Library.swapaxes(lib, 0, 1)
    assert sw.dim_names == ['y', 'x'] and sw.shape == (3, 4)
    np.testing.assert_array_equal(sw['f'], lib['f'].T)
    with pytest.raises(ValueError):
        Library.swapaxes(Library(Dimension('x', [0., 1.])), 0, 0)


def test_scale_and_remap_dimension():
    lib = _lib2()
    lib.scale_dimension('x', 2.)
    np.testing.assert_allclose(lib.x_values, np.linspace(0, 2, 4))
    np.testing.assert_allclose(lib.x_grid[:, 0], np.linspace(0, 2, 4))
    lib.remap_dimension('y', lambda v: v + 1.)
    np.testing.assert_allclose(lib.y_values, np.linspace(0, 2, 3))
    with pytest.raises(KeyError):
        lib.scale_dimension('z', 2.)


@pytest.mark.parametrize('ndim', [1, 2, 3])
def test_pickle_round_trip(tmp_path, ndim):
    dims = [Dimension(n, np.linspace(0, 1, k)) for n, k in zip('xyz', (16, 8, 4))][:ndim]
    l1 = Library(*dims)
    l1['f'] = sum(getattr(l1, n + '_grid') for n in 'xyz'[:ndim])
    l1['g'] = np.exp(l1['f'])
    l1.extra_attributes['name'] = 'my_library_name'
    p = str(tmp_path / 'lib.pkl')
    l1.save_to_file(p)
    l2 = Library.load_from_file(p)
    assert l2.dim_names == l1.dim_names
    for q in ('f', 'g'):
        np.testing.assert_array_equal(l2[q], l1[q])
    assert l2.extra_attributes['name'] == 'my_library_name'


def test_text_directory(tmp_path):
    lib = _lib2()
    lib['with space'] = lib['f'] * 2.
    out = str(tmp_path / 'txt')
    lib.save_to_text_directory(out)
    with open(os.path.join(out, 'metadata_independent_variables.txt')) as f:
        assert f.read().split() == ['x', 'y']
    with open(os.path.join(out, 'metadata_dependent_variables.txt')) as f:
        assert f.read().split() == ['f', 'g', 'with_space']
    np.testing.assert_allclose(np.loadtxt(os.path.join(out, 'bulkdata_ivar_y.txt')), lib.y_values)
    np.testing.assert_allclose(np.loadtxt(os.path.join(out, 'bulkdata_dvar_with_space.txt')),
                               lib['with space'].ravel(order='F'), rtol=1e-13)
    with pytest.raises(FileExistsError):
        lib.save_to_text_directory(out)
    lib.save_to_text_directory(out, ravel_order='C', overwrite=True)
    np.testing.assert_allclose(np.loadtxt(os.path.join(out, 'bulkdata_dvar_f.txt')), lib['f'].ravel(order='C'),
                               rtol=1e-13)


GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')


@pytest.mark.parametrize('name,dims,shape', [('adiabatic_slfm', ['mixture_fraction', 'dissipation_rate_stoich'], (34, 8)),
                                             ('nonadiabatic_defect_burke_schumann',
                                              ['mixture_fraction', 'enthalpy_defect_stoich'], (34, 16))])
def test_reads_reference_written_library(name, dims, shape):
    """A library the reference pickled (its tests/tabulation gold files, copied unchanged) loads into this
    package's Library, with its dimensions, properties and mechanism."""
    from spitfire_gb300.mechanism import ChemicalMechanismSpec
    lib = Library.load_from_file(os.path.join(GOLD, f'reference_{name}_gold.pkl'))
    assert isinstance(lib, Library)
    assert lib.dim_names == dims and lib.shape == shape
    assert lib['temperature'].shape == shape
    assert np.all(lib['temperature'] > 250.) and np.allclose(lib['pressure'], 101325., rtol=1e-12)
    ys = sum(lib[p] for p in lib.props if p.startswith('mass fraction '))
    assert np.allclose(ys, 1., atol=1e-10)
    mech = lib.extra_attributes['mech_spec']
    assert isinstance(mech, ChemicalMechanismSpec) and mech.n_species == 11
    if name == 'adiabatic_slfm':
        g = np.load(os.path.join(GOLD, 'adiabatic_slfm_gold.npz'))
        np.testing.assert_array_equal(lib['temperature'], g['prop:temperature'])
        np.testing.assert_array_equal(lib.dissipation_rate_stoich_values, g['dim1_values'])
    # a reference library saved again by this package reads back the same
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, 'again.pkl')
        lib.save_to_file(p)
        lib2 = Library.load_from_file(p)
    np.testing.assert_array_equal(lib2['temperature'], lib['temperature'])
    assert lib2.extra_attributes['mech_spec'].n_species == 11
