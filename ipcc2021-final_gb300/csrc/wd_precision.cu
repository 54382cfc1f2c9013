// wd_precision.cu -- derived copies of the resident links.
#include "wd_precision.h"

void wd_lattice_invalidate_derived(wd_lattice *lat)
{
    cudaFree(lat->gauge_df);
    cudaFree(lat->gauge_f32);
    cudaFree(lat->gauge_h12);
    lat->gauge_df = nullptr;
    lat->gauge_f32 = nullptr;
    lat->gauge_h12 = nullptr;
}
