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
//     unless constructed with one); fence() synchronises that stream.
#pragma once

#include <cuda_runtime.h>

#include <array>
#include <cstddef>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>

#define KOKKOS_FUNCTION
#define KOKKOS_INLINE_FUNCTION inline

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
        constexpr std::size_t se[] = {Exts...};
        for (std::size_t r = 0; r < rank(); ++r) {
            m_ext[r] = se[r] == dynamic_extent ? 0 : static_cast<IndexType>(se[r]);
        }
    }

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

template <class T>
struct default_accessor
{
    using element_type = T;
    using reference = T&;
    using data_handle_type = T*;
};

// Non-owning multidimensional view over contiguous memory (host-side index
// arithmetic only; the kernels receive data_handle() pointers).
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
        std::int64_t const ix[] = {static_cast<std::int64_t>(idx)...};
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
        return m_ptr[off];
    }

private:
    data_handle_type m_ptr = nullptr;
    Extents m_ext {};
};

// Declared only: the reference's subspan helpers are templates nobody
// instantiates in the operator path.
template <class... Args>
void submdspan(Args const&...) = delete;

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
