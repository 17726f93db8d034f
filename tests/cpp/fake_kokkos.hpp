// A stand-in for the part of Kokkos that the drop-in headers meet (test
// only): Kokkos::View<T *, Device> with data(), extent(i) and stride(i)
// over device memory, and KOKKOS_VERSION, which the headers test for.  Lets
// the C++ drop-in test compile the Kokkos form of
// PointCloudOperator<DeviceType>::apply without a Kokkos installation.
#pragma once
#include <cstddef>

#define KOKKOS_VERSION 40100

namespace Kokkos
{
template <class DataType, class Device>
struct View;

template <class T, class Device>
struct View<T *, Device>
{
    T *ptr = nullptr;
    std::size_t n = 0;
    View() = default;
    View( T *p, std::size_t count )
        : ptr( p )
        , n( count )
    {
    }
    // a view of non-const values converts to a view of const values
    template <class U>
    View( View<U *, Device> const &o )
        : ptr( o.ptr )
        , n( o.n )
    {
    }
    T *data() const { return ptr; }
    std::size_t extent( int d ) const { return d == 0 ? n : 1; }
    std::ptrdiff_t stride( int ) const { return 1; }
};
} // namespace Kokkos
