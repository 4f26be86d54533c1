"""GB300-native GetHI realisation path (damonge/CRIME drop-in for
create_d_and_vr_fields -> get_HI -> mk_T_maps; see crime_gb300.gethi) and the
JoinT map combination that consumes its maps (see crime_gb300.joint)."""
from .gethi import (GetHI, GetHIError, Params, default_params, host_modes_mt, host_psources, host_setup, make_params,
                    read_params, read_run_params, run_batch)
from .joint import JoinT

__all__ = ["GetHI", "GetHIError", "Params", "default_params", "host_modes_mt", "host_psources", "host_setup",
           "make_params",
           "read_params", "read_run_params", "run_batch", "JoinT"]
