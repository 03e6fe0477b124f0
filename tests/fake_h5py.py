"""In-memory stand-in for the part of h5py that the monitors use, for
machines without h5py: File (modes 'w', 'a', 'r'; context manager; attrs),
groups (create_group, require_group, item access by name or path),
datasets (create_dataset with shape / dtype / data and the compression
arguments, slice assignment with casting to the dataset's dtype).

As h5py, a dataset created from a shape alone stores float32.  Files live
in the module-level FILES table until ``reset()``; ``snapshot(name)``
describes a file as plain data (attributes, and per dataset its shape,
dtype, compression and contents) for comparisons."""
import numpy as np

FILES = {}


def reset():
    FILES.clear()


class Dataset(object):
    def __init__(self, shape=None, dtype=None, data=None, compression=None,
                 compression_opts=None):
        if data is not None:
            data = np.asarray(data)
            arr = np.array(data, dtype=dtype or data.dtype)
            if shape is not None and tuple(shape) != arr.shape:
                raise ValueError('shape %r does not match the data %r'
                                 % (shape, arr.shape))
        else:
            if shape is None:
                raise TypeError('create_dataset needs a shape or data')
            arr = np.zeros(tuple(shape), dtype=dtype or np.float32)
        self._a = arr
        self.compression = compression
        self.compression_opts = compression_opts

    @property
    def shape(self):
        return self._a.shape

    @property
    def dtype(self):
        return self._a.dtype

    def __getitem__(self, key):
        return np.array(self._a[key])

    def __setitem__(self, key, value):
        self._a[key] = np.asarray(value)


class Group(object):
    def __init__(self):
        self._items = {}

    def _walk(self, path, create=False):
        node = self
        parts = [p for p in path.split('/') if p]
        for p in parts[:-1]:
            node = node._items[p]
        return node, parts[-1]

    def create_group(self, name):
        node, leaf = self._walk(name)
        if leaf in node._items:
            raise ValueError('name already exists: %s' % name)
        g = Group()
        node._items[leaf] = g
        return g

    def require_group(self, name):
        node, leaf = self._walk(name)
        if leaf in node._items:
            g = node._items[leaf]
            if not isinstance(g, Group):
                raise TypeError('%s is not a group' % name)
            return g
        return self.create_group(name)

    def create_dataset(self, name, shape=None, dtype=None, data=None,
                       compression=None, compression_opts=None, **kwargs):
        if kwargs:
            raise TypeError('unsupported create_dataset arguments %r'
                            % sorted(kwargs))
        node, leaf = self._walk(name)
        if leaf in node._items:
            raise ValueError('name already exists: %s' % name)
        d = Dataset(shape, dtype, data, compression, compression_opts)
        node._items[leaf] = d
        return d

    def __getitem__(self, name):
        node, leaf = self._walk(name)
        return node._items[leaf]

    def __contains__(self, name):
        try:
            self[name]
            return True
        except KeyError:
            return False

    def keys(self):
        return list(self._items)


class _FileData(Group):
    def __init__(self):
        Group.__init__(self)
        self.attrs = {}


class File(object):
    def __init__(self, name, mode='r'):
        if mode == 'w':
            FILES[name] = _FileData()
        elif mode == 'a':
            FILES.setdefault(name, _FileData())
        elif mode == 'r':
            if name not in FILES:
                raise IOError('no such file: %s' % name)
        else:
            raise ValueError('mode %r' % mode)
        self.name = name
        self._f = FILES[name]
        self.attrs = self._f.attrs

    def __getattr__(self, name):
        return getattr(self._f, name)

    def __getitem__(self, name):
        return self._f[name]

    def __contains__(self, name):
        return name in self._f

    def close(self):
        pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
        return False


def snapshot(name):
    """{'attrs': {key: value}, 'datasets': {path: {'shape', 'dtype',
    'compression', 'compression_opts', 'data'}}, 'groups': [paths]}."""
    f = FILES[name]
    out = {'attrs': dict(f.attrs), 'datasets': {}, 'groups': []}

    def walk(g, prefix):
        for k, v in g._items.items():
            path = prefix + k
            if isinstance(v, Group):
                out['groups'].append(path)
                walk(v, path + '/')
            else:
                out['datasets'][path] = {
                    'shape': list(v.shape), 'dtype': v.dtype.str,
                    'compression': v.compression,
                    'compression_opts': v.compression_opts,
                    'data': np.array(v._a)}
    walk(f, '')
    out['groups'].sort()
    return out
