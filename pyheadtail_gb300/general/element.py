"""Printing and Element base classes with PyHEADTAIL's contract
(general/element.py:16-85): every element offers ``track(beam)``; output goes
through the ``printer`` / ``warningprinter`` keyword arguments."""
from abc import ABCMeta, abstractmethod

from .printers import ConsolePrinter


class Printing(object):
    """Gives ``prints`` / ``warns`` with a pluggable Printer."""

    def __init__(self, *args, **kwargs):
        pass

    def __new__(cls, *args, **kwargs):
        instance = object.__new__(cls)
        instance._printer = kwargs.get('printer', ConsolePrinter())
        instance._warningprinter = kwargs.get('warningprinter',
                                              ConsolePrinter())
        return instance

    def prints(self, output):
        self._printer.prints(output)

    def warns(self, output):
        self._warningprinter.prints('*** PyHEADTAIL WARNING! ' + output)


class Element(Printing, metaclass=ABCMeta):
    """A tracking element: ``track(beam)`` advances the beam through it."""

    @abstractmethod
    def track(self, beam):
        pass
