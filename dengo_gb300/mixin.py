"""``ComparableMixin`` (reference: dengo/mixin.py:5-34): total order, equality
and hash of the network objects through their ``_cmpkey``."""

from .reaction_classes import ComparableMixin  # noqa: F401
