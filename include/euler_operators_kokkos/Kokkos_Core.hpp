// Kokkos names for builds of the euler_operators drop-in WITHOUT Kokkos.
//
// The operator headers in include/euler_operators/ keep the reference's
// signatures, which name Kokkos::mdspan, Kokkos::extents, Kokkos::layout_left,
// Kokkos::View and Kokkos::DefaultExecutionSpace.  With a real Kokkos (CUDA
// backend) on the include path those come from Kokkos itself.  Without one,
// put this directory on the include path: it supplies the handful of names
// the reference's driver and operators use, backed by CUDA:
//   * View<T*> allocates CUDA managed memory (cudaMallocManaged, preferred
//     location the current device), so kernels and host code (the driver's
//     NPY output, simulations/euler_simulation.cpp:71-79) can both read it;
//   * DefaultExecutionSpace wraps a cudaStream_t (the legacy default stream
//     unless constructed with one); fence() synchronises that stream;
//   * mdspan (layout_left, layout_right, layout_stride) with submdspan over
//     index, full_extent and [first, last) pair slices, for the bundles'
//     subspan helpers.
#pragma once

#include <cuda_runtime.h>

#include <array>
#include <cstddef>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <tuple>
#include <type_traits>
#include <utility>

// As with Kokkos's CUDA backend, KOKKOS_FUNCTION code is callable from the
// device when nvcc compiles it.
#if defined(__CUDACC__)
#define KOKKOS_FUNCTION __host__ __device__
#define KOKKOS_INLINE_FUNCTION __host__ __device__ inline
#else
#define KOKKOS_FUNCTION
#define KOKKOS_INLINE_FUNCTION inline
#endif

namespace Kokkos {

inline constexpr std::size_t dynamic_extent = static_cast<std::size_t>(-1);

template <class IndexType, std::size_t... Exts>
class extents
{
public:
    using index_type = IndexType;
    using size_type = std::make_unsigned_t<IndexType>;
    using rank_type = std::size_t;

    static constexpr rank_type rank() noexcept { return sizeof...(Exts); }

    constexpr extents() noexcept
    {
        if constexpr (sizeof...(Exts) > 0) {
            constexpr std::size_t se[] = {Exts...};
            for (std::size_t r = 0; r < rank(); ++r) {
                m_ext[r] = se[r] == dynamic_extent ? 0 : static_cast<IndexType>(se[r]);
            }
        }
    }

    template <class... I,
              class = std::enable_if_t<sizeof...(I) == sizeof...(Exts) && (std::is_integral_v<I> && ...)>>
    constexpr explicit extents(I... e) noexcept : m_ext {static_cast<IndexType>(e)...}
    {
    }

    template <class OI>
    constexpr explicit extents(std::array<OI, sizeof...(Exts)> const& e) noexcept
    {
        for (std::size_t r = 0; r < rank(); ++r) {
            m_ext[r] = static_cast<IndexType>(e[r]);
        }
    }

    template <class OI, std::size_t... OE>
    constexpr extents(extents<OI, OE...> const& o) noexcept
    {
        for (std::size_t r = 0; r < rank(); ++r) {
            m_ext[r] = static_cast<IndexType>(o.extent(r));
        }
    }

    constexpr index_type extent(rank_type r) const noexcept { return m_ext[r]; }

private:
    std::array<IndexType, sizeof...(Exts)> m_ext {};
};

namespace detail {
template <class I, std::size_t R, std::size_t... D>
struct dextents_of : dextents_of<I, R - 1, dynamic_extent, D...>
{
};
template <class I, std::size_t... D>
struct dextents_of<I, 0, D...>
{
    using type = extents<I, D...>;
};
} // namespace detail

template <class IndexType, std::size_t Rank>
using dextents = typename detail::dextents_of<IndexType, Rank>::type;

struct layout_left
{
};
struct layout_right
{
};
// Any strides: what submdspan returns where a slice is not one contiguous
// block of the parent.
struct layout_stride
{
};

template <class T>
struct default_accessor
{
    using element_type = T;
    using reference = T&;
    using data_handle_type = T*;
};

// Non-owning multidimensional view (host-side index arithmetic only; the
// kernels receive data_handle() pointers).  layout_left and layout_right
// views are contiguous, their strides follow from the extents; a
// layout_stride view carries its own.
template <class T, class Extents, class Layout = layout_right, class Accessor = default_accessor<T>>
class mdspan
{
public:
    using element_type = T;
    using value_type = std::remove_cv_t<T>;
    using extents_type = Extents;
    using layout_type = Layout;
    using accessor_type = Accessor;
    using index_type = typename Extents::index_type;
    using rank_type = typename Extents::rank_type;
    using data_handle_type = typename Accessor::data_handle_type;
    using reference = typename Accessor::reference;
    using strides_type = std::array<index_type, Extents::rank()>;

    mdspan() = default;

    template <class... I, class = std::enable_if_t<(std::is_integral_v<I> && ...)>>
    mdspan(data_handle_type p, I... exts) noexcept : m_ptr(p), m_ext(exts...)
    {
        static_assert(!std::is_same_v<Layout, layout_stride>, "a layout_stride view needs its strides");
        set_contiguous_strides();
    }

    mdspan(data_handle_type p, Extents const& e) noexcept : m_ptr(p), m_ext(e)
    {
        static_assert(!std::is_same_v<Layout, layout_stride>, "a layout_stride view needs its strides");
        set_contiguous_strides();
    }

    mdspan(data_handle_type p, Extents const& e, strides_type const& strides) noexcept
        : m_ptr(p), m_ext(e), m_stride(strides)
    {
        static_assert(std::is_same_v<Layout, layout_stride>, "only a layout_stride view takes strides");
    }

    template <class OT, class OE, class OA>
    mdspan(mdspan<OT, OE, Layout, OA> const& o) noexcept : m_ptr(o.data_handle()), m_ext(o.extents())
    {
        for (std::size_t r = 0; r < rank(); ++r) {
            m_stride[r] = static_cast<index_type>(o.stride(r));
        }
    }

    static constexpr rank_type rank() noexcept { return Extents::rank(); }
    index_type extent(rank_type r) const noexcept { return m_ext.extent(r); }
    index_type stride(rank_type r) const noexcept { return m_stride[r]; }
    Extents const& extents() const noexcept { return m_ext; }
    data_handle_type data_handle() const noexcept { return m_ptr; }

    std::size_t size() const noexcept
    {
        std::size_t s = 1;
        for (std::size_t r = 0; r < rank(); ++r) {
            s *= static_cast<std::size_t>(m_ext.extent(r));
        }
        return s;
    }

    template <class... I>
    reference operator()(I... idx) const noexcept
    {
        static_assert(sizeof...(I) == Extents::rank());
        std::int64_t off = 0;
        if constexpr (sizeof...(I) > 0) {
            std::int64_t const ix[] = {static_cast<std::int64_t>(idx)...};
            for (std::size_t r = 0; r < rank(); ++r) {
                off += ix[r] * static_cast<std::int64_t>(m_stride[r]);
            }
        }
        return m_ptr[off];
    }

private:
    void set_contiguous_strides() noexcept
    {
        index_type s = 1;
        if constexpr (std::is_same_v<Layout, layout_left>) {
            for (std::size_t r = 0; r < rank(); ++r) {
                m_stride[r] = s;
                s *= m_ext.extent(r);
            }
        } else {
            for (std::size_t r = rank(); r-- > 0;) {
                m_stride[r] = s;
                s *= m_ext.extent(r);
            }
        }
    }

    data_handle_type m_ptr = nullptr;
    Extents m_ext {};
    strides_type m_stride {};
};

// Slice specifiers of submdspan: an index (the rank is dropped), full_extent,
// or a half-open range [first, last) as a std::pair or a two-element
// std::tuple.
struct full_extent_t
{
    explicit full_extent_t() = default;
};
inline constexpr full_extent_t full_extent {};
// Kokkos's own spellings of these slices
inline constexpr full_extent_t ALL {};
template <class A, class B>
using pair = std::pair<A, B>;
using std::make_pair;

namespace detail {
enum class slice_kind { index, full, range };

template <class S>
struct slice_traits
{
    static_assert(std::is_integral_v<S>, "a slice is an index, full_extent or a [first, last) pair");
    static constexpr slice_kind kind = slice_kind::index;
    template <class I>
    static std::array<std::int64_t, 2> bounds(S const& s, I /*extent*/) noexcept
    {
        return {static_cast<std::int64_t>(s), 1};
    }
};

template <>
struct slice_traits<full_extent_t>
{
    static constexpr slice_kind kind = slice_kind::full;
    template <class I>
    static std::array<std::int64_t, 2> bounds(full_extent_t const&, I extent) noexcept
    {
        return {0, static_cast<std::int64_t>(extent)};
    }
};

template <class A, class B>
struct slice_traits<std::pair<A, B>>
{
    static constexpr slice_kind kind = slice_kind::range;
    template <class I>
    static std::array<std::int64_t, 2> bounds(std::pair<A, B> const& s, I /*extent*/) noexcept
    {
        return {static_cast<std::int64_t>(s.first), static_cast<std::int64_t>(s.second) - static_cast<std::int64_t>(s.first)};
    }
};

template <class A, class B>
struct slice_traits<std::tuple<A, B>>
{
    static constexpr slice_kind kind = slice_kind::range;
    template <class I>
    static std::array<std::int64_t, 2> bounds(std::tuple<A, B> const& s, I /*extent*/) noexcept
    {
        return {static_cast<std::int64_t>(std::get<0>(s)),
                static_cast<std::int64_t>(std::get<1>(s)) - static_cast<std::int64_t>(std::get<0>(s))};
    }
};

// Whether the slices of a layout_left view leave one contiguous block with
// i fastest: the kept ranks come first, all but the last of them whole.
// layout_right mirrors it (kept ranks last, all but the first whole).
template <class... S>
constexpr bool keeps_contiguous(bool left) noexcept
{
    constexpr slice_kind k[] = {slice_traits<S>::kind..., slice_kind::index};
    constexpr std::size_t n = sizeof...(S);
    std::size_t kept = 0;
    for (std::size_t r = 0; r < n; ++r) {
        kept += k[r] != slice_kind::index ? 1 : 0;
    }
    for (std::size_t q = 0; q < kept; ++q) {
        std::size_t const r = left ? q : n - kept + q;
        bool const edge = left ? q + 1 == kept : q == 0;
        if (k[r] == slice_kind::index || (!edge && k[r] != slice_kind::full)) {
            return false;
        }
    }
    return true;
}
} // namespace detail

// The part of a view that the slices select (C++26 std::submdspan,
// restricted to the slice forms above); the result has dynamic extents.
template <class T, class E, class L, class A, class... S>
auto submdspan(mdspan<T, E, L, A> const& m, S const&... slices)
{
    static_assert(sizeof...(S) == E::rank(), "one slice per rank");
    using I = typename E::index_type;
    constexpr std::size_t rank_out = ((detail::slice_traits<S>::kind != detail::slice_kind::index ? 1 : 0) + ... + 0);
    constexpr bool contiguous = (std::is_same_v<L, layout_left> && detail::keeps_contiguous<S...>(true))
                                || (std::is_same_v<L, layout_right> && detail::keeps_contiguous<S...>(false));
    using layout_out = std::conditional_t<contiguous, L, layout_stride>;
    using extents_out = dextents<I, rank_out>;
    std::array<I, rank_out> ext {};
    std::array<I, rank_out> str {};
    std::int64_t off = 0;
    std::size_t r = 0;
    std::size_t q = 0;
    auto one = [&](auto const& s) {
        using traits = detail::slice_traits<std::remove_cv_t<std::remove_reference_t<decltype(s)>>>;
        std::array<std::int64_t, 2> const b = traits::bounds(s, m.extent(r));
        off += b[0] * static_cast<std::int64_t>(m.stride(r));
        if constexpr (traits::kind != detail::slice_kind::index) {
            ext[q] = static_cast<I>(b[1]);
            str[q] = m.stride(r);
            ++q;
        }
        ++r;
    };
    (one(slices), ...);
    if constexpr (contiguous) {
        return mdspan<T, extents_out, layout_out, A>(m.data_handle() + off, extents_out(ext));
    } else {
        return mdspan<T, extents_out, layout_out, A>(m.data_handle() + off, extents_out(ext), str);
    }
}

class DefaultExecutionSpace
{
public:
    DefaultExecutionSpace() noexcept = default;
    explicit DefaultExecutionSpace(cudaStream_t s) noexcept : m_stream(s) {}
    cudaStream_t cuda_stream() const noexcept { return m_stream; }
    void fence() const
    {
        cudaError_t const e = cudaStreamSynchronize(m_stream);
        if (e != cudaSuccess) {
            throw std::runtime_error(std::string("fence: ") + cudaGetErrorString(e));
        }
    }

private:
    cudaStream_t m_stream = nullptr;
};

class ScopeGuard
{
public:
    ScopeGuard(int& /*argc*/, char** /*argv*/) { cudaFree(nullptr); }
    ~ScopeGuard() { cudaDeviceSynchronize(); }
    ScopeGuard(ScopeGuard const&) = delete;
    ScopeGuard& operator=(ScopeGuard const&) = delete;
};

struct ViewAllocProp
{
    std::string label;
};

inline ViewAllocProp view_alloc(DefaultExecutionSpace const& /*exec*/, std::string label)
{
    return {std::move(label)};
}

template <class DataType>
class View;

// Owning 1D array in CUDA managed memory, zero-initialised like a Kokkos View.
template <class T>
class View<T*>
{
public:
    View() = default;
    View(ViewAllocProp const& prop, std::size_t n) : m_label(prop.label), m_size(n)
    {
        void* p = nullptr;
        cudaError_t e = cudaMallocManaged(&p, n * sizeof(T) > 0 ? n * sizeof(T) : 1);
        if (e != cudaSuccess) {
            throw std::runtime_error("View " + m_label + ": " + cudaGetErrorString(e));
        }
        int dev = 0;
        cudaGetDevice(&dev);
        cudaMemLocation loc {};
        loc.type = cudaMemLocationTypeDevice;
        loc.id = dev;
        cudaMemAdvise(p, n * sizeof(T), cudaMemAdviseSetPreferredLocation, loc);
        cudaMemset(p, 0, n * sizeof(T));
        m_data = std::shared_ptr<T[]>(static_cast<T*>(p), [](T* q) { cudaFree(q); });
    }
    T* data() const noexcept { return m_data.get(); }
    std::size_t size() const noexcept { return m_size; }
    std::size_t extent(std::size_t /*r*/) const noexcept { return m_size; }
    std::string const& label() const noexcept { return m_label; }

private:
    std::shared_ptr<T[]> m_data;
    std::string m_label;
    std::size_t m_size = 0;
};

using std::max;
using std::min;

} // namespace Kokkos
