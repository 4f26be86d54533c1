"""GB300-native GetHI realisation path (damonge/CRIME drop-in for
create_d_and_vr_fields -> get_HI -> mk_T_maps).  See crime_gb300.gethi."""
from .gethi import (GetHI, GetHIError, Params, default_params, host_modes_mt, host_psources, host_setup, make_params,
                    read_params, read_run_params, run_batch)

__all__ = ["GetHI", "GetHIError", "Params", "default_params", "host_modes_mt", "host_psources", "host_setup",
           "make_params",
           "read_params", "read_run_params", "run_batch"]
