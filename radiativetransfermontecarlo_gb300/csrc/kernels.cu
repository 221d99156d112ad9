// Instantiation unit of the transport kernel family (transport.cuh).  The build compiles
// this file eight times, once per precision RTMC_REAL (float, double) and part RTMC_PART
// (1 the transport kernels, 2 the batched kernels, 3 the adjoint kernels, 4 the kernels of
// the split schedule), so the variants compile in parallel; RTMC_SUFFIX names the
// precision (f32, f64).
#include "transport.cuh"

#if !defined(RTMC_REAL) || !defined(RTMC_PART) || !defined(RTMC_SUFFIX)
#error "compile with -DRTMC_REAL=float|double -DRTMC_SUFFIX=f32|f64 -DRTMC_PART=1|2|3|4"
#endif

#define RTMC_CAT2(a, b) a##_##b
#define RTMC_CAT(a, b) RTMC_CAT2(a, b)
#define RTMC_NAME(n) RTMC_CAT(n, RTMC_SUFFIX)

namespace rtmc {

#if RTMC_PART == 1
int RTMC_NAME(launch_transport)(const DevParams<RTMC_REAL> &p, int grid, int block, size_t smem, void *stream)
{
    return launch_transport_t<RTMC_REAL>(p, grid, block, smem, stream);
}

void *RTMC_NAME(kernel_of_transport)(int sink, int obs) { return pick_t<RTMC_REAL>(sink, obs); }
#elif RTMC_PART == 4
int RTMC_NAME(launch_split)(const DevParams<RTMC_REAL> &p, const SplitLaunch &l, void *stream)
{
    return launch_split_t<RTMC_REAL>(p, l, stream);
}

void *RTMC_NAME(kernel_of_split)(int kind, int sink, int obs)
{
    return kind == 5 ? pick_events<RTMC_REAL>(obs) : (kind == 6 ? pick_observe<RTMC_REAL>(sink, obs) : pick_list<RTMC_REAL>(sink, obs));
}
#elif RTMC_PART == 2
int RTMC_NAME(launch_transport_batch)(const BatchArgs<RTMC_REAL> &a, int grid, int block, size_t smem, void *stream,
                                      int split)
{
    return launch_batch_t<RTMC_REAL>(a, grid, block, smem, stream, split ? 2 : 0);
}

int RTMC_NAME(launch_transport_batch_em)(const BatchArgs<RTMC_REAL> &a, int grid, int block, size_t smem, void *stream,
                                         int shist)
{
    return launch_batch_t<RTMC_REAL>(a, grid, block, smem, stream, shist ? 3 : 1);
}

void *RTMC_NAME(kernel_of_batch)(int which, int obs) { return pick_batch_kind<RTMC_REAL>(which, obs); }
#elif RTMC_PART == 3
int RTMC_NAME(launch_adjoint)(const DevParams<RTMC_REAL> &p, const AdjointArgs &a, int grid, int block, size_t smem,
                              void *stream)
{
    return launch_adjoint_t<RTMC_REAL>(p, a, grid, block, smem, stream, false);
}

int RTMC_NAME(launch_adjoint_ring)(const DevParams<RTMC_REAL> &p, const AdjointArgs &a, int grid, int block, size_t smem,
                                   void *stream)
{
    return launch_adjoint_t<RTMC_REAL>(p, a, grid, block, smem, stream, true);
}

void *RTMC_NAME(kernel_of_adjoint)(int which, int obs)
{
    switch (which) {
    case 0: return pick_adjoint<RTMC_REAL>(obs);
    case 1: return pick_adjoint_ring<RTMC_REAL>(obs);
    case 2: return pick_observe_adj<RTMC_REAL>(obs);
    default: return pick_adjoint_list<RTMC_REAL>(obs);
    }
}
#endif

} // namespace rtmc
