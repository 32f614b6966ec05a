"""dpx — GB300-native scattering hot path of D+ (amplitude grid, docked sum,
orientation average) behind the libdpx C-ABI."""
from ._lib import DpxError, lib, EXPORTED  # noqa: F401
from .models import (Context, Grid, PDBAmplitude, calculate_grids, autotune_fill, pdb_descs, SolveBatch, AmpGridAmplitude, read_amp, ManualSymmetry, SpaceFillingSymmetry, DomainModel,  # noqa: F401
                     FP32, FP64,
                     mc_directions, layer_seeds, layer_directions, make_globule)
from . import state  # noqa: F401,E402
