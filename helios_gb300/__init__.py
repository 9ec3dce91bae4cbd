"""helios_gb300 -- GB300-native closed-shell PPP CCSD (helios ``r-ccsd``).

The engine is the CUDA library ``_lib/libhelios_gb300.so`` (built by
``python -m helios_gb300.build``) behind the C ABI ``include/helios_cc.h``;
``api`` mirrors helios's coupled-cluster routines over it, ``molecules``
generates the PPP inputs. Around the path: ``properties`` (the polarizability
job), ``lrccsd`` (LR-CCSD excited states), ``inputfile`` (helios input files),
``replicas`` (independent molecules over several GPUs).
"""
from .molecules import Molecule, polyene, ladder, dodecahexaene, random_molecule, ensemble  # noqa: F401

__all__ = ["Molecule", "polyene", "ladder", "dodecahexaene", "random_molecule", "ensemble"]
