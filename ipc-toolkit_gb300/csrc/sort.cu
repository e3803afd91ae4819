// sort.cu — radix sort / run-length / unique primitives (CUB device
// algorithms), kept in one translation unit so the template instantiations
// are compiled once.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_run_length_encode.cuh>
#include <cub/device/device_scan.cuh>
#include <cub/device/device_select.cuh>

#include "internal.cuh"
#include "profile.cuh"

namespace ipcg {

namespace {
// CUB device calls are timed and counted as one launch each.
// The temporary storage is the mesh's; calls on one mesh are stream ordered
// (its main stream, or its side stream with the main stream waiting).
template <typename F> void with_temp(ipcg_mesh* m, cudaStream_t st, const char* name, F&& f)
{
    size_t bytes = 0;
    IPCG_CUDA(f(nullptr, bytes));
    m->tmp.reserve(bytes + 256);
    bytes = m->tmp.cap;
    IPCG_LAUNCH(name, st, IPCG_CUDA(f((void*)m->tmp.p, bytes)));
}
} // namespace

void sort_pairs_u32(ipcg_mesh* m, cudaStream_t st, const unsigned* k_in, unsigned* k_out, const int* v_in, int* v_out, int n,
    int end_bit)
{
    if (n <= 0) return;
    with_temp(m, st, "cub_radix_sort_pairs", [&](void* t, size_t& b) {
        return cub::DeviceRadixSort::SortPairs(t, b, k_in, k_out, v_in, v_out, n, 0, end_bit, st);
    });
}

void sort_keys_u64(ipcg_mesh* m, cudaStream_t st, const unsigned long long* k_in, unsigned long long* k_out, int n, int end_bit)
{
    if (n <= 0) return;
    with_temp(m, st, "cub_radix_sort_keys", [&](void* t, size_t& b) {
        return cub::DeviceRadixSort::SortKeys(t, b, k_in, k_out, n, 0, end_bit, st);
    });
}

void sort_pairs_u64(ipcg_mesh* m, cudaStream_t st, const unsigned long long* k_in, unsigned long long* k_out, const int* v_in,
    int* v_out, int n, int end_bit)
{
    if (n <= 0) return;
    with_temp(m, st, "cub_radix_sort_pairs", [&](void* t, size_t& b) {
        return cub::DeviceRadixSort::SortPairs(t, b, k_in, k_out, v_in, v_out, n, 0, end_bit, st);
    });
}

void rle_u64(ipcg_mesh* m, cudaStream_t st, const unsigned long long* k_in, unsigned long long* uniq, int* counts, int* d_num, int n)
{
    if (n <= 0) {
        IPCG_CUDA(cudaMemsetAsync(d_num, 0, sizeof(int), st));
        return;
    }
    with_temp(m, st, "cub_run_length_encode", [&](void* t, size_t& b) {
        return cub::DeviceRunLengthEncode::Encode(t, b, k_in, uniq, counts, d_num, n, st);
    });
}

void unique_u64(ipcg_mesh* m, cudaStream_t st, const unsigned long long* k_in, unsigned long long* uniq, int* d_num, int n)
{
    if (n <= 0) {
        IPCG_CUDA(cudaMemsetAsync(d_num, 0, sizeof(int), st));
        return;
    }
    with_temp(m, st, "cub_select_unique", [&](void* t, size_t& b) {
        return cub::DeviceSelect::Unique(t, b, k_in, uniq, d_num, n, st);
    });
}

void exclusive_sum_i64(ipcg_mesh* m, cudaStream_t st, const int64_t* in, int64_t* out, int n)
{
    if (n <= 0) return;
    with_temp(m, st, "cub_exclusive_sum", [&](void* t, size_t& b) {
        return cub::DeviceScan::ExclusiveSum(t, b, in, out, n, st);
    });
}

void exclusive_sum_i32(ipcg_mesh* m, cudaStream_t st, const int* in, int* out, int n)
{
    if (n <= 0) return;
    with_temp(m, st, "cub_exclusive_sum", [&](void* t, size_t& b) {
        return cub::DeviceScan::ExclusiveSum(t, b, in, out, n, st);
    });
}

} // namespace ipcg
