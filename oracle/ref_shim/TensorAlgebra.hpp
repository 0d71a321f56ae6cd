// GRTeclyn header stand-in (test infrastructure): nothing from it is used by
// the hot-path headers compiled here.
#pragma once
#include "axs_amrex_shim.H"
