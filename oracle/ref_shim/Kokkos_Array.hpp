// Project-written stand-in for Kokkos::Array (an aggregate fixed-size array).
#ifndef DTK_REF_SHIM_KOKKOS_ARRAY_HPP
#define DTK_REF_SHIM_KOKKOS_ARRAY_HPP

#include "Kokkos_Macros.hpp"

#include <cstddef>

namespace Kokkos
{
template <class T, size_t N>
struct Array
{
    T _data[N];
    T &operator[]( size_t i ) { return _data[i]; }
    T const &operator[]( size_t i ) const { return _data[i]; }
    static constexpr size_t size() { return N; }
    T *data() { return _data; }
    T const *data() const { return _data; }
};
} // namespace Kokkos

#endif
