"""Ideal transverse damper (feedback/transverse_damper.py:15-94).

The reference measures the bunch's dipole moment with ``mean_xp()`` (and
``mean_x()`` for a reactive damper) and subtracts a fraction of it from
every particle's xp.  Here ``track(beam)`` does both on the device without
a host sync:

1. one statistics pass (``phk_bunch_stats``, order 1, over xp / yp and x / y
   when reactive) of the beam's state, with pending wake kicks applied in
   registers, writes the bunch means to a device buffer of this damper;
2. a DAMPER op is appended to the beam's pending program: the next fused
   pass subtracts ``(g sin(phase)) <xp>`` (then ``((g cos(phase)) <x>) /
   beta``) from every xp, reading the means from that buffer, in the
   reference's order of operations.
"""
import weakref

import numpy as np
import torch

from .. import _engine as E
from .. import _native as N
from ..general.element import Element
from ..particles import statistics as S


class TransverseDamper(Element):

    def __init__(self, dampingrate_x, dampingrate_y, phase=90,
                 local_beta_function=None, *args, **kwargs):
        """Same arguments as the reference (transverse_damper.py:17-62):
        damping rates in turns (0 or None: plane off), the kick phase in
        degrees with respect to the pick-up, and the local beta function
        (required unless the phase is 90 or 270 degrees)."""
        self.gain_x = self.gain_y = None
        if dampingrate_x and not dampingrate_y:
            self.gain_x = 2 / dampingrate_x
            self.prints('Damper in horizontal plane active')
        elif not dampingrate_x and dampingrate_y:
            self.gain_y = 2 / dampingrate_y
            self.prints('Damper in vertical plane active')
        elif not dampingrate_x and not dampingrate_y:
            self.prints('Dampers not active')
        else:
            self.gain_x = 2 / dampingrate_x
            self.gain_y = 2 / dampingrate_y
            self.prints('Dampers active')
        if phase != 90 and phase != 270 and not local_beta_function:
            raise TypeError(
                'TransverseDamper: numeric local_beta_function value at '
                'position of damper missing! (Required because of non-zero '
                'reactive damper component.)')
        self.phase_in_2pi = phase / 360. * 2 * np.pi
        self.local_beta_function = local_beta_function
        # per beam: the statistics record and the means buffer the op reads
        self._bufs = weakref.WeakKeyDictionary()

    @classmethod
    def horizontal(cls, dampingrate_x, *args, **kwargs):
        return cls(dampingrate_x, 0, *args, **kwargs)

    @classmethod
    def vertical(cls, dampingrate_y, *args, **kwargs):
        return cls(0, dampingrate_y, *args, **kwargs)

    def _op(self, means, gains):
        flags, p = 0, {}
        coords = ()
        for pl, gain in ((0, gains[0]), (1, gains[1])):
            if gain is None:
                continue
            flags |= N.FLAG_DAMP_X if pl == 0 else N.FLAG_DAMP_Y
            u, up = ('x', 'xp') if pl == 0 else ('y', 'yp')
            coords += (up,)
            # the reference's scalars: gain * sin(phase), gain * cos(phase)
            p[3 * pl] = gain * np.sin(self.phase_in_2pi)
            p[3 * pl + 1] = gain * np.cos(self.phase_in_2pi)
            p[3 * pl + 2] = (float(self.local_beta_function)
                             if self.local_beta_function else 1.0)
            if self.local_beta_function:
                coords += (u,)
        if self.local_beta_function:
            flags |= N.FLAG_REACTIVE
        pf = {k: np.float32(v) for k, v in p.items()}
        # the means pointer goes to the eight bytes of p[31]
        return (E.Op(N.OP_DAMPER, flags, p=p, pf=pf,
                     pointer=means.data_ptr()), S.mask_of(coords))

    def track(self, beam):
        """transverse_damper.py:64-86: the planes whose damping rate is
        set (the reference binds track to track_horizontal, _vertical or
        _all), deferred to the beam's next pass."""
        self._track_planes(beam, (self.gain_x, self.gain_y))

    def track_horizontal(self, beam):
        """transverse_damper.py:68-72."""
        self._track_planes(beam, (self._gain('x'), None))

    def track_vertical(self, beam):
        """transverse_damper.py:74-78."""
        self._track_planes(beam, (None, self._gain('y')))

    def track_all(self, beam):
        """transverse_damper.py:80-88."""
        self._track_planes(beam, (self._gain('x'), self._gain('y')))

    def _gain(self, plane):
        g = self.gain_x if plane == 'x' else self.gain_y
        if g is None:
            # the reference's arithmetic on an unset gain fails the same way
            raise TypeError('TransverseDamper: no damping rate in the %s '
                            'plane' % plane)
        return g

    def _track_planes(self, beam, gains):
        if gains[0] is None and gains[1] is None:
            return
        buf = self._bufs.get(beam)
        if buf is None:
            buf = (torch.zeros(S.RECORD_LEN, dtype=torch.float64,
                               device=beam._device),
                   torch.zeros(9, dtype=torch.float64, device=beam._device))
            self._bufs[beam] = buf
        rec, means = buf
        op, mask = self._op(means, gains)
        op.keepalive = means        # referenced by pointer until the pass
        beam.launch_stats(rec, order=1, mask=mask, means=means)
        beam._engine.enqueue(op)
