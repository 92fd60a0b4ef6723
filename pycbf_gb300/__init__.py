"""pycbf_gb300: GB300-native (sm_103a) drop-in for pycbf's beamforming hot path.

The classes mirror pycbf.gpu / pycbf.cpu (TabbedBeamformer, SyntheticBeamformer,
TabbedDMASBeamformer, SyntheticDMASBeamformer) and add SLSC beamformers.  All
compute runs in hand-written CUDA kernels of libpycbf_gb300.so, called through
its C ABI (include/pycbf_gb300.h); there is no CPU fallback.
"""
from .beamformers import (Beamformer, BeamformerException, DMASBeamformer, Synthetic,
                          SyntheticBeamformer, SyntheticDMASBeamformer, SyntheticSLSCBeamformer,
                          Tabbed, TabbedBeamformer, TabbedDMASBeamformer, TabbedSLSCBeamformer)

__all__ = ["Beamformer", "BeamformerException", "DMASBeamformer", "Synthetic",
           "SyntheticBeamformer", "SyntheticDMASBeamformer", "SyntheticSLSCBeamformer", "Tabbed",
           "TabbedBeamformer", "TabbedDMASBeamformer", "TabbedSLSCBeamformer"]
