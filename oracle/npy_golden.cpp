// Test-only: writes small arrays with the reference's own NPY writer
// (simulations/save_npy.{hpp,cpp}, compiled unmodified through the test-only
// Kokkos shim) so the GB300 driver's writer can be checked byte for byte.
//   npy_golden <out_dir>   ->  npy_ref_f64.npy (3x4x5, layout_left), npy_ref_f32.npy (2x3x2)
#include <string>
#include <vector>

#include <Kokkos_Core.hpp>

#include "save_npy.hpp"

int main(int argc, char** argv)
{
    std::string const dir = argc > 1 ? argv[1] : ".";
    std::vector<double> a(3 * 4 * 5);
    for (int k = 0; k < 5; ++k) {
        for (int j = 0; j < 4; ++j) {
            for (int i = 0; i < 3; ++i) {
                a[i + 3 * (j + 4 * k)] = i + 10.0 * j + 100.0 * k + 0.25;
            }
        }
    }
    Kokkos::mdspan<double, Kokkos::dextents<int, 3>, Kokkos::layout_left> va(a.data(), 3, 4, 5);
    save_npy(std::filesystem::path(dir + "/npy_ref_f64.npy"), va);
    std::vector<float> b(2 * 3 * 2);
    for (std::size_t i = 0; i < b.size(); ++i) {
        b[i] = 0.5f * static_cast<float>(i) - 1.0f;
    }
    Kokkos::mdspan<float, Kokkos::dextents<int, 3>, Kokkos::layout_left> vb(b.data(), 2, 3, 2);
    save_npy(std::filesystem::path(dir + "/npy_ref_f32.npy"), vb);
    return 0;
}
