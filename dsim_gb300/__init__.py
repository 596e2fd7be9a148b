"""GB300-native engine for dSim's Monte-Carlo diffusion-MRI hot path.

Native libraries (built in-tree by dsim_gb300.build):
  libdsim_gb300.so  native C-ABI (include/dsim.h)
  libdsim3.so       drop-in for the reference's dSim3 plugin boundary
  libdsim2.so       drop-in for the reference's dSim2 plugin boundary
"""
__version__ = "0.1.0"
