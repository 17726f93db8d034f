// Project-written stand-in for the Kokkos macros used by the DataTransferKit
// MLS numerics headers (host-only checker build).
#ifndef DTK_REF_SHIM_KOKKOS_MACROS_HPP
#define DTK_REF_SHIM_KOKKOS_MACROS_HPP

#define KOKKOS_INLINE_FUNCTION inline
#define KOKKOS_FUNCTION
#define KOKKOS_DEFAULTED_FUNCTION
#define KOKKOS_LAMBDA [=]

#endif
