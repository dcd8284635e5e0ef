"""neuwon_gb300: GB300-native (sm_103a) implementation of NEUWON's Model.advance() hot path.

The host API mirrors the reference's RxD_Model / Neuron / Segment / Mechanism
interface; every time step runs in hand-written CUDA kernels behind the C ABI
declared in include/neuwon_gb300.h (loaded with ctypes, no CPU fallback).
"""
from .kinetic import Kinetic, KineticScheme, Kv11, LTITable, Nav11, kv11, na8, nav11
from .mechanisms import HH, Mechanism, NMODL
from .model import Clock, Model, Neuron, RxD_Model, Segment, TimeSeries
from .morphology import EPSILON, Tree, geometry, neuron_sizes, passive_electric, random_tree
from .species import Calcium, SpeciesType
from .synapses import SynapseKinetics

__all__ = ["Kinetic", "KineticScheme", "LTITable", "na8", "nav11", "kv11", "Nav11", "Kv11", "HH", "Mechanism",
           "NMODL", "Clock", "Model", "Neuron", "RxD_Model", "Segment", "TimeSeries", "EPSILON", "Tree", "geometry",
           "neuron_sizes", "passive_electric", "random_tree", "Calcium", "SpeciesType", "SynapseKinetics"]
__version__ = "0.2.0"
