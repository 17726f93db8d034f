// Minimal host-only stand-in for the subset of the Kokkos API that the
// DataTransferKit MLS numerics headers use, written for this project so that
// those headers (SVD, MLS Impl, RBF, polynomial basis) compile unchanged with
// g++ as a test-only checker.  It is not Kokkos: Views are reference-counted
// host arrays (LayoutRight, zero-initialised), parallel_for / parallel_reduce
// run an OpenMP loop, fence() is a no-op.
#ifndef DTK_REF_SHIM_KOKKOS_CORE_HPP
#define DTK_REF_SHIM_KOKKOS_CORE_HPP

#include "Kokkos_Macros.hpp"
#include "Kokkos_Array.hpp"

#include <cfloat>
#include <cmath>
#include <cstddef>
#include <memory>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

namespace Kokkos
{

struct HostSpace
{
};
struct Serial
{
    using execution_space = Serial;
    using memory_space = HostSpace;
};
template <class Exec, class Mem>
struct Device
{
    using execution_space = Exec;
    using memory_space = Mem;
};

template <class T1, class T2>
struct pair
{
    T1 first;
    T2 second;
};
template <class T1, class T2>
KOKKOS_INLINE_FUNCTION pair<T1, T2> make_pair( T1 a, T2 b )
{
    return pair<T1, T2>{a, b};
}

struct ALL_t
{
    ALL_t operator()() const { return *this; }
};
constexpr ALL_t ALL{};

template <class DataType, class... Props>
class View;

// Rank-1 view.
template <class T, class... Props>
class View<T *, Props...>
{
  public:
    using value_type = T;
    using non_const_value_type = std::remove_const_t<T>;
    using const_type = View<const non_const_value_type *, Props...>;
    using non_const_type = View<non_const_value_type *, Props...>;
    static constexpr int rank = 1;

    View() = default;
    View( std::string const &label, size_t n )
        : _store( std::make_shared<std::vector<non_const_value_type>>( n ) )
        , _ptr( _store->data() )
        , _n( n )
        , _label( label )
    {
    }
    template <class U, class... Q,
              class = std::enable_if_t<std::is_same<
                  const std::remove_const_t<U>, const non_const_value_type>::value>>
    View( View<U *, Q...> const &o )
        : _store( o._store )
        , _ptr( o._ptr )
        , _n( o._n )
        , _label( o._label )
    {
    }

    T &operator()( size_t i ) const { return _ptr[i]; }
    T &operator[]( size_t i ) const { return _ptr[i]; }
    T &access( size_t i, size_t = 0 ) const { return _ptr[i]; }
    size_t extent( int d ) const { return d == 0 ? _n : 1; }
    int extent_int( int d ) const { return (int)extent( d ); }
    size_t size() const { return _n; }
    T *data() const { return _ptr; }
    std::string label() const { return _label; }

    std::shared_ptr<std::vector<non_const_value_type>> _store;
    T *_ptr = nullptr;
    size_t _n = 0;
    std::string _label;
};

// Rank-2 view (row-major with explicit strides so that column sub-ranges of
// a wider array keep their original row stride).
template <class T, class... Props>
class View<T **, Props...>
{
  public:
    using value_type = T;
    using non_const_value_type = std::remove_const_t<T>;
    using const_type = View<const non_const_value_type **, Props...>;
    using non_const_type = View<non_const_value_type **, Props...>;
    static constexpr int rank = 2;

    View() = default;
    View( std::string const &label, size_t n0, size_t n1 )
        : _store( std::make_shared<std::vector<non_const_value_type>>( n0 * n1 ) )
        , _ptr( _store->data() )
        , _n0( n0 )
        , _n1( n1 )
        , _s0( n1 )
        , _label( label )
    {
    }
    template <class U, class... Q,
              class = std::enable_if_t<std::is_same<
                  const std::remove_const_t<U>, const non_const_value_type>::value>>
    View( View<U **, Q...> const &o )
        : _store( o._store )
        , _ptr( o._ptr )
        , _n0( o._n0 )
        , _n1( o._n1 )
        , _s0( o._s0 )
        , _label( o._label )
    {
    }

    T &operator()( size_t i, size_t j ) const { return _ptr[i * _s0 + j]; }
    T &access( size_t i, size_t j = 0 ) const { return _ptr[i * _s0 + j]; }
    size_t extent( int d ) const { return d == 0 ? _n0 : d == 1 ? _n1 : 1; }
    int extent_int( int d ) const { return (int)extent( d ); }
    T *data() const { return _ptr; }
    std::string label() const { return _label; }

    std::shared_ptr<std::vector<non_const_value_type>> _store;
    T *_ptr = nullptr;
    size_t _n0 = 0, _n1 = 0, _s0 = 0;
    std::string _label;
};

template <class T, class... P, class I>
View<T *, P...> subview( View<T *, P...> const &v, pair<I, I> r )
{
    View<T *, P...> out = v;
    out._ptr = v._ptr + r.first;
    out._n = (size_t)( r.second - r.first );
    return out;
}

template <class T, class... P, class I>
View<T **, P...> subview( View<T **, P...> const &v, ALL_t, pair<I, I> r )
{
    View<T **, P...> out = v;
    out._ptr = v._ptr + r.first;
    out._n1 = (size_t)( r.second - r.first );
    return out;
}

template <class Exec = Serial>
struct RangePolicy
{
    RangePolicy( long b, long e )
        : begin( b )
        , end( e )
    {
    }
    long begin, end;
};

template <class Policy, class F>
void parallel_for( std::string const &, Policy const &p, F const &f )
{
#pragma omp parallel for schedule( dynamic, 64 )
    for ( long i = p.begin; i < p.end; ++i )
        f( (int)i );
}

template <class Policy, class F, class R>
void parallel_reduce( std::string const &, Policy const &p, F const &f, R &result )
{
    R acc = 0;
#pragma omp parallel for schedule( dynamic, 16 ) reduction( + : acc )
    for ( long i = p.begin; i < p.end; ++i )
        f( (int)i, acc );
    result = acc;
}

inline void fence() {}

} // namespace Kokkos

#endif
