// GRTeclyn header stand-in (test infrastructure): the parity enum that
// StateVariables.hpp names (periodic runs never use it).
#pragma once
enum class BCParity
{
    even,
    odd
};
