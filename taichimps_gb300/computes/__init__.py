from .thermo import BOLTZMANN, Computes, virial_chunks

__all__ = ["Computes", "virial_chunks", "BOLTZMANN"]
