/*
 * Per-thread views of shared-memory arrays laid out [slot][lanes]: thread
 * tid's slot i is p[i * LANES], so a warp's accesses are conflict-free.
 */
#ifndef DG_SLOTS_CUH
#define DG_SLOTS_CUH

namespace dg {

/* One double per thread and slot. */
template <int LANES>
struct Slots {
    double *p;
    __device__ __forceinline__ double &operator[](int i) const { return p[i * LANES]; }
};

/* One float per thread and slot (the mixed path's FP32 factors). */
template <int LANES>
struct SlotsF {
    float *p;
    __device__ __forceinline__ float &operator[](int i) const { return p[i * LANES]; }
};

}  // namespace dg
#endif
