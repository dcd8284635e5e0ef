"""neuwon_gb300: GB300-native (sm_103a) implementation of NEUWON's Model.advance() hot path.

The host API mirrors the reference's RxD_Model / Neuron / Segment / Mechanism
interface; every time step runs in hand-written CUDA kernels behind the C ABI
declared in include/neuwon_gb300.h (loaded with ctypes, no CPU fallback).
"""
from .kinetic import (NMDA, Kinetic, KineticScheme, KineticScheme2, Kv11, LTITable, LTITable2, Nav11, TableInput,
                      kv11, na8, nav11, nmda)
from .mechanisms import HH, Mechanism, NMODL
from .model import Clock, Model, Neuron, RxD_Model, Segment, TimeSeries
from .morphology import EPSILON, Tree, geometry, neuron_sizes, passive_electric, random_tree
from .species import Calcium, SpeciesType
from .synapses import SynapseKinetics

__all__ = ["Kinetic", "KineticScheme", "KineticScheme2", "LTITable", "LTITable2", "TableInput", "na8", "nav11",
           "kv11", "nmda", "Nav11", "Kv11", "NMDA", "HH", "Mechanism",
           "NMODL", "Clock", "Model", "Neuron", "RxD_Model", "Segment", "TimeSeries", "EPSILON", "Tree", "geometry",
           "neuron_sizes", "passive_electric", "random_tree", "Calcium", "SpeciesType", "SynapseKinetics"]
__version__ = "0.2.0"
