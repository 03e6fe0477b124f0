"""Output channels for Printing, mirroring PyHEADTAIL's general/printers.py
(Printer :12-31, ConsolePrinter :34-44, SilentPrinter :47-55,
AccumulatorPrinter :58-67)."""
from abc import ABCMeta, abstractmethod


class Printer(object, metaclass=ABCMeta):
    """Where a Printing object sends its text."""

    @abstractmethod
    def prints(self, output):
        pass


class ConsolePrinter(Printer):
    def prints(self, output):
        print(output)


class SilentPrinter(Printer):
    def prints(self, output):
        pass


class AccumulatorPrinter(Printer):
    """Keeps every message in ``self.log`` (used by tests)."""

    def __init__(self, *args, **kwargs):
        self.log = []

    def prints(self, output):
        self.log.append(output)
