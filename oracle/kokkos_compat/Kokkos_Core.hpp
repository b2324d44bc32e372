// Test-only Kokkos compatibility layer for the CPU oracle.
//
// This is test infrastructure, not product code: it exists so that the
// reference's header-only operators (euler_operators/*.hpp) compile unmodified
// with plain g++ and OpenMP, producing the reference build that pins the C restatement
// in oracle/euler_oracle.c.  It implements only the subset of the Kokkos API
// those headers touch:
//   mdspan / extents / dextents / layout_left / layout_right / default_accessor
//   View<T*> + view_alloc, MDRangePolicy<Rank<3,...>, IndexType<I>>,
//   parallel_for, parallel_reduce with Min<T>, Array<T,N>, min/max/abs/sqrt,
//   KOKKOS_FUNCTION / KOKKOS_LAMBDA, DefaultExecutionSpace::fence, ScopeGuard,
//   and a declaration of submdspan (used only by uninstantiated templates).
// Iteration order follows Iterate::Left (i fastest).  OpenMP splits the
// (k, j) rows among the threads, as Kokkos's OpenMP MDRangePolicy tiles more
// than the outermost axis; the only reduction is an exact min, so results do not
// depend on the thread count.
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <limits>
#include <memory>
#include <string>
#include <type_traits>
#include <utility>

#define KOKKOS_FUNCTION
#define KOKKOS_INLINE_FUNCTION inline
#define KOKKOS_LAMBDA [=]

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

    static constexpr std::size_t static_extent(rank_type r) noexcept
    {
        constexpr std::size_t se[] = {Exts...};
        return se[r];
    }

    constexpr extents() noexcept
    {
        constexpr std::size_t se[] = {Exts...};
        for (std::size_t r = 0; r < rank(); ++r) {
            m_ext[r] = se[r] == dynamic_extent ? 0 : static_cast<IndexType>(se[r]);
        }
    }

    // One value per extent (the oracle only builds fully dynamic extents).
    template <class... I, class = std::enable_if_t<sizeof...(I) == sizeof...(Exts)>>
    constexpr explicit extents(I... e) noexcept : m_ext {static_cast<IndexType>(e)...}
    {
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
struct dextents_helper : dextents_helper<I, R - 1, dynamic_extent, D...>
{
};
template <class I, std::size_t... D>
struct dextents_helper<I, 0, D...>
{
    using type = extents<I, D...>;
};
} // namespace detail

template <class IndexType, std::size_t Rank>
using dextents = typename detail::dextents_helper<IndexType, Rank>::type;

struct layout_left
{
};
struct layout_right
{
};

template <class T>
struct default_accessor
{
    using element_type = T;
    using reference = T&;
    using data_handle_type = T*;
    using offset_policy = default_accessor;
};

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
    using size_type = typename Extents::size_type;
    using rank_type = typename Extents::rank_type;
    using data_handle_type = typename Accessor::data_handle_type;
    using reference = typename Accessor::reference;

    mdspan() = default;

    template <class... I>
    mdspan(data_handle_type p, I... exts) noexcept : m_ptr(p), m_ext(exts...)
    {
    }

    template <class OT, class OE, class OA>
    mdspan(mdspan<OT, OE, Layout, OA> const& o) noexcept : m_ptr(o.data_handle()), m_ext(o.extents())
    {
    }

    static constexpr rank_type rank() noexcept { return Extents::rank(); }

    index_type extent(rank_type r) const noexcept { return m_ext.extent(r); }
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
        return m_ptr[offset(static_cast<std::int64_t>(idx)...)];
    }

private:
    template <class... I>
    std::int64_t offset(I... idx) const noexcept
    {
        std::int64_t const ix[] = {idx...};
        std::int64_t off = 0;
        if constexpr (std::is_same_v<Layout, layout_left>) {
            for (std::size_t r = rank(); r-- > 0;) {
                off = off * m_ext.extent(r) + ix[r];
            }
        } else {
            for (std::size_t r = 0; r < rank(); ++r) {
                off = off * m_ext.extent(r) + ix[r];
            }
        }
        return off;
    }

    data_handle_type m_ptr = nullptr;
    Extents m_ext {};
};

// Only referenced from templates the oracle never instantiates.
template <class... Args>
void submdspan(Args const&...) = delete;

template <class T, std::size_t N>
struct Array
{
    T m_internal_implementation_private_member_data[N];
    constexpr T& operator[](std::size_t i) noexcept
    {
        return m_internal_implementation_private_member_data[i];
    }
    constexpr T const& operator[](std::size_t i) const noexcept
    {
        return m_internal_implementation_private_member_data[i];
    }
};

template <class T>
constexpr T const& min(T const& a, T const& b) noexcept
{
    return (b < a) ? b : a;
}

template <class T>
constexpr T const& max(T const& a, T const& b) noexcept
{
    return (a < b) ? b : a;
}

using std::abs;
using std::sqrt;

struct DefaultExecutionSpace
{
    void fence() const noexcept {}
};

class ScopeGuard
{
public:
    ScopeGuard(int& /*argc*/, char** /*argv*/) noexcept {}
    ScopeGuard(ScopeGuard const&) = delete;
    ScopeGuard& operator=(ScopeGuard const&) = delete;
};

struct ViewAllocLabel
{
    std::string label;
};

inline ViewAllocLabel view_alloc(DefaultExecutionSpace const& /*exec*/, std::string label)
{
    return {std::move(label)};
}

template <class DataType>
class View;

template <class T>
class View<T*>
{
public:
    View() = default;
    View(ViewAllocLabel const& /*alloc*/, std::size_t n) : m_data(new T[n]()), m_size(n) {}
    T* data() const noexcept { return m_data.get(); }
    std::size_t size() const noexcept { return m_size; }
    std::size_t extent(std::size_t /*r*/) const noexcept { return m_size; }
    T& operator()(std::size_t i) const noexcept { return m_data[i]; }

private:
    std::shared_ptr<T[]> m_data;
    std::size_t m_size = 0;
};

struct Iterate
{
    struct Left
    {
    };
    struct Right
    {
    };
};

template <unsigned N, class OuterIter = Iterate::Left, class InnerIter = Iterate::Left>
struct Rank
{
    static constexpr unsigned rank = N;
};

template <class I>
struct IndexType
{
    using type = I;
};

template <class RankT, class IndexT>
struct MDRangePolicy
{
    static_assert(RankT::rank == 3, "the oracle only iterates 3D ranges");
    using index_type = typename IndexT::type;

    MDRangePolicy(
            DefaultExecutionSpace const& /*exec*/,
            std::array<std::int64_t, 3> const& lo,
            std::array<std::int64_t, 3> const& hi) noexcept
        : begin(lo)
        , end(hi)
    {
    }

    std::array<std::int64_t, 3> begin;
    std::array<std::int64_t, 3> end;
};

template <class T>
struct Min
{
    explicit Min(T& result) noexcept : ref(result) {}
    T& ref;
};

template <class RankT, class IndexT, class F>
void parallel_for(std::string const& /*label*/, MDRangePolicy<RankT, IndexT> const& p, F const& f)
{
    using I = typename IndexT::type;
#pragma omp parallel for collapse(2) schedule(static)
    for (std::int64_t k = p.begin[2]; k < p.end[2]; ++k) {
        for (std::int64_t j = p.begin[1]; j < p.end[1]; ++j) {
            for (std::int64_t i = p.begin[0]; i < p.end[0]; ++i) {
                f(static_cast<I>(i), static_cast<I>(j), static_cast<I>(k));
            }
        }
    }
}

template <class RankT, class IndexT, class F, class T>
void parallel_reduce(
        std::string const& /*label*/,
        MDRangePolicy<RankT, IndexT> const& p,
        F const& f,
        Min<T> reducer)
{
    using I = typename IndexT::type;
    T global = std::numeric_limits<T>::max();
#pragma omp parallel
    {
        T local = std::numeric_limits<T>::max();
#pragma omp for collapse(2) schedule(static)
        for (std::int64_t k = p.begin[2]; k < p.end[2]; ++k) {
            for (std::int64_t j = p.begin[1]; j < p.end[1]; ++j) {
                for (std::int64_t i = p.begin[0]; i < p.end[0]; ++i) {
                    f(static_cast<I>(i), static_cast<I>(j), static_cast<I>(k), local);
                }
            }
        }
#pragma omp critical
        {
            if (local < global) {
                global = local;
            }
        }
    }
    reducer.ref = global;
}

} // namespace Kokkos
