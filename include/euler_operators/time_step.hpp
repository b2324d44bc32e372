// euler_operators drop-in for GB300: time_step, the reference's
// euler_operators/time_step.hpp:8-41 -- min over all cells of
// 1 / sum_d (c + |u_d|) / dx_d, without the CFL factor.  Reduced on the GPU by
// eulr_time_step_{f64,f32} (bit-identical to the reference) into a device
// scalar of the calling thread on the current device (one per thread and
// device, allocated on first use and kept until the process exits), then
// copied back: like the reference, it returns a host value and therefore
// waits for the execution space's stream.
#pragma once

#include <map>

#include <euler_arrays.hpp>
#include <euler_gb300_bridge.hpp>
#include <perfect_gas.hpp>
#include <uniform_mesh.hpp>

template <class T, class IndexType, std::size_t E0, std::size_t E1, std::size_t E2>
T time_step(
        Kokkos::DefaultExecutionSpace const& exec_space,
        EulerPrimArrays<Kokkos::mdspan<T const, Kokkos::extents<IndexType, E0, E1, E2>, Kokkos::layout_left>> const&
                prim_arrays,
        PerfectGas<T> const& eos,
        UniformMesh3d<T> const& mesh)
{
    namespace b = euler_gb300_bridge;
    using ty = b::types<T>;
    // the result slot of this thread on the current device: the reduction
    // must write to memory of the device it runs on
    static thread_local std::map<int, T*> dt_dev_of;
    int dev = 0;
    cudaError_t const de = cudaGetDevice(&dev);
    if (de != cudaSuccess) {
        throw std::runtime_error(std::string("time_step: ") + cudaGetErrorString(de));
    }
    T*& dt_dev = dt_dev_of[dev];
    if (dt_dev == nullptr) {
        cudaError_t const e = cudaMalloc(&dt_dev, sizeof(T));
        if (e != cudaSuccess) {
            dt_dev = nullptr;
            throw std::runtime_error(std::string("time_step: ") + cudaGetErrorString(e));
        }
    }
    auto const& s = prim_arrays.d;
    eulr_stream_t const stream = b::stream_of(exec_space);
    int st;
    if constexpr (std::is_same_v<T, double>) {
        st = eulr_time_step_f64(b::prim_ptrs<typename ty::cprim>(prim_arrays), b::extent_int(s, 0), b::extent_int(s, 1),
                                b::extent_int(s, 2), eos.gamma(), mesh.dx0(), mesh.dx1(), mesh.dx2(), dt_dev, stream);
    } else {
        st = eulr_time_step_f32(b::prim_ptrs<typename ty::cprim>(prim_arrays), b::extent_int(s, 0), b::extent_int(s, 1),
                                b::extent_int(s, 2), eos.gamma(), mesh.dx0(), mesh.dx1(), mesh.dx2(), dt_dev, stream);
    }
    b::check(st, "time_step");
    T dt {};
    cudaError_t e = cudaMemcpyAsync(&dt, dt_dev, sizeof(T), cudaMemcpyDeviceToHost, exec_space.cuda_stream());
    if (e == cudaSuccess) {
        e = cudaStreamSynchronize(exec_space.cuda_stream());
    }
    if (e != cudaSuccess) {
        throw std::runtime_error(std::string("time_step: ") + cudaGetErrorString(e));
    }
    return dt;
}
