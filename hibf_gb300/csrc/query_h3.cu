// query_h3.cu -- the HIBF query kernels for hierarchies with 3 hash function(s): every tuning variant and the
// learned scheduler's feature kernel.
// One translation unit per hash function count keeps the instantiations compiling in parallel.
#include "query.cuh"

namespace hibf_gb300
{
query_kernel_t query_kernel_h3(int v)
{
    return query_kernel_variant<3>(v);
}
query_kernel_t query_block_kernel_h3()
{
    return k_query_blk<3>;
}
features_kernel_t features_kernel_h3()
{
    return k_query_features<3>;
}
} // namespace hibf_gb300
