from .contact_atom import ComputeContactAtom
from .thermo import BOLTZMANN, Computes, virial_chunks

__all__ = ["Computes", "ComputeContactAtom", "virial_chunks", "BOLTZMANN"]
