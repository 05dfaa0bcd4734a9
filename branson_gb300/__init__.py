"""branson_gb300: Branson's replicated-mode IMC transport step on GB300 (sm_103a).

The compute path is the shared library built from csrc/ (C ABI in
include/branson_gb300.h); this package is its host-side mirror: the deck
model (deck.py), the ctypes binding (_lib.py) and the replicated driver
(engine.py).
"""
from . import deck
from .deck import Deck, load as load_deck, parse_xml
from ._lib import BransonError, PhotonArrays, HISTORY, EVENT

__all__ = ["deck", "Deck", "load_deck", "parse_xml", "BransonError", "PhotonArrays", "HISTORY", "EVENT",
           "ReplicatedIMC"]


def __getattr__(name):
    if name == "ReplicatedIMC":
        from .engine import ReplicatedIMC
        return ReplicatedIMC
    raise AttributeError(name)
