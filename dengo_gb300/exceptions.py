"""Exceptions of the network-definition API (reference: dengo/exceptions.py).

The lookups of unknown reaction, cooling-action and species names raise
these; they also derive from ``KeyError``, the error a registry lookup
raises, so either can be caught."""


class DengoException(Exception):
    pass


class UnknownReaction(DengoException, KeyError):
    def __init__(self, name):
        super().__init__(name)
        self.name = name

    def __str__(self):
        return "Dengo doesn't know about reaction %s" % (self.name,)


class UnknownSpecies(DengoException, KeyError):
    def __init__(self, name):
        super().__init__(name)
        self.name = name

    def __str__(self):
        return "Dengo doesn't know about species %s" % (self.name,)


class UnknownCoolingAction(DengoException, KeyError):
    def __init__(self, name):
        super().__init__(name)
        self.name = name

    def __str__(self):
        return "Dengo doesn't know about cooling action %s" % (self.name,)
