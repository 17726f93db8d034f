// Project-written stand-in for DTK's generated configuration header (the
// checker build enables design-by-contract checks).
#ifndef DTK_REF_SHIM_CONFIG_HPP
#define DTK_REF_SHIM_CONFIG_HPP
#define HAVE_DTK_DBC 1
#endif
