"""Record the HDF5 layout the reference's monitors write, without h5py.

Run in a container where the reference source tree is present:

    python tests/golden/make_golden_monitors.py --ref <PyHEADTAIL source tree>

The reference's BunchMonitor, SliceMonitor and ParticleMonitor
(monitors/monitors.py:39-470) are driven through the runs of
monitor_cases.py with an in-memory h5py stand-in (tests/fake_h5py.py)
installed as ``h5py``; the bunches are host objects that return the
cases' values.  Every file's attributes, groups and datasets (shape,
dtype, compression, contents) go to monitors/layout.npz, which the host
test of this repository's monitors compares against.
"""
import argparse
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(HERE))
import make_golden as MG  # noqa: E402
import monitor_cases as MC  # noqa: E402
import fake_h5py  # noqa: E402

OUT = os.path.join(HERE, 'monitors', 'layout.npz')


class StatsBunch(object):
    """Bunch statistics as methods, the macroparticle number as an
    attribute, slices through get_slices: the values of ``step``."""

    def __init__(self, n_slices=None):
        self.step = 0
        self.n_slices = n_slices

    @property
    def macroparticlenumber(self):
        return MC.bunch_value('macroparticlenumber', self.step)

    def get_slices(self, slicer, statistics=None):
        ss = type('SliceSetValues', (), {})()
        ss.n_slices = self.n_slices
        for st in MC.SLICE_STATS:
            setattr(ss, st, MC.slice_value(st, self.step, self.n_slices))
        return ss


for _st in MC.BUNCH_STATS:
    if _st != 'macroparticlenumber':
        setattr(StatsBunch, _st,
                (lambda s: lambda self: MC.bunch_value(s, self.step))(_st))


class CoordBunch(object):
    def __init__(self, step, n):
        self.arrays, self.extra = MC.particle_arrays(step, n)
        self.macroparticlenumber = n
        for k, v in self.arrays.items():
            setattr(self, k, v)

    def get_coords_n_momenta_dict(self):
        return {k: self.arrays[k] for k in MC.COORDS[:-1]}


def pack(snapshots):
    meta, arrays = {}, {}
    for fname, snap in snapshots.items():
        m = {'attrs': snap['attrs'], 'groups': snap['groups'],
             'datasets': {}}
        for path, d in snap['datasets'].items():
            m['datasets'][path] = {k: v for k, v in d.items() if k != 'data'}
            arrays['data::%s::%s' % (fname, path)] = d['data']
        meta[fname] = m
    return meta, arrays


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--ref', required=True,
                    help='PyHEADTAIL source tree (read only)')
    ap.add_argument('--scratch', default='/tmp/phk_refbuild')
    a = ap.parse_args()
    MG.build_reference(a.ref, a.scratch)
    sys.modules['h5py'] = fake_h5py
    from PyHEADTAIL.monitors import monitors as RM
    from PyHEADTAIL.general.printers import SilentPrinter
    fake_h5py.reset()

    r = MC.BUNCH_RUN
    bunch = StatsBunch()
    mon = RM.BunchMonitor('bunch', r['n_steps'], dict(MC.PARAMETERS),
                          write_buffer_every=r['write_buffer_every'],
                          buffer_size=r['buffer_size'],
                          printer=SilentPrinter())
    for step in range(r['n_steps']):
        bunch.step = step
        mon.dump(bunch)

    r = MC.SLICE_RUN
    bunch = StatsBunch(r['n_slices'])
    slicer = type('SlicerShape', (), {'n_slices': r['n_slices']})()
    mon = RM.SliceMonitor('slices', r['n_steps'], slicer,
                          dict(MC.PARAMETERS),
                          write_buffer_every=r['write_buffer_every'],
                          buffer_size=r['buffer_size'],
                          printer=SilentPrinter())
    for step in range(r['n_steps']):
        bunch.step = step
        mon.dump(bunch)

    r = MC.PARTICLE_RUN
    mon = RM.ParticleMonitor('particles', stride=r['stride'],
                             parameters_dict=dict(MC.PARAMETERS),
                             printer=SilentPrinter())
    for step in range(r['n_dumps']):
        b = CoordBunch(step, r['n'])
        mon.dump(b, arrays_dict=b.extra)

    snaps = {name: fake_h5py.snapshot(name)
             for name in ('bunch.h5', 'slices.h5', 'particles.h5part')}
    meta, arrays = pack(snaps)
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    np.savez_compressed(OUT, __meta__=np.array(json.dumps(meta, default=str)),
                        **arrays)
    print('wrote', OUT, sorted(meta))


if __name__ == '__main__':
    main()
