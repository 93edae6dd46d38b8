// query_h2.cu -- the HIBF query kernels for hierarchies with 2 hash function(s): every tuning variant and the
// learned scheduler's feature kernel.
// One translation unit per hash function count keeps the instantiations compiling in parallel.
#include "query.cuh"

namespace hibf_gb300
{
query_kernel_t query_kernel_h2(int v)
{
    return query_kernel_variant<2>(v);
}
query_kernel_t query_block_kernel_h2()
{
    return k_query_blk<2>;
}
features_kernel_t features_kernel_h2()
{
    return k_query_features<2>;
}
} // namespace hibf_gb300
