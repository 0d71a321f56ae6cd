// GRTeclyn header stand-in (test infrastructure).
#pragma once
#include "axs_amrex_shim.H"
