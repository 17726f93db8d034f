// Project-written stand-in for the few ArborX names that the DataTransferKit
// MLS numerics headers touch outside the search itself (ArborX is not
// vendored with the reference).  Points hold doubles, matching DTK's
// Coordinate = double; distance() is the Euclidean distance accumulated over
// d = 0, 1, 2 from zero.  The neighbour search is not provided here: the
// checker driver takes its connectivity from the oracle's exact kNN.
#ifndef DTK_REF_SHIM_ARBORX_HPP
#define DTK_REF_SHIM_ARBORX_HPP

#include "Kokkos_Core.hpp"

#include <cmath>

namespace ArborX
{
struct Point
{
    double _coords[3];
    double &operator[]( int i ) { return _coords[i]; }
    double const &operator[]( int i ) const { return _coords[i]; }
};

template <class Geometry>
struct Nearest
{
    Geometry geometry;
    int k;
};

inline Nearest<Point> nearest( Point const &p, int k ) { return {p, k}; }

namespace Details
{
inline double distance( Point const &a, Point const &b )
{
    double acc = 0.0;
    for ( int d = 0; d < 3; ++d )
    {
        double const t = b[d] - a[d];
        acc += t * t;
    }
    return std::sqrt( acc );
}
} // namespace Details

template <class T, class... P>
T lastElement( Kokkos::View<T *, P...> const &v )
{
    return v.extent( 0 ) ? v( v.extent( 0 ) - 1 ) : T{};
}
} // namespace ArborX

#endif
