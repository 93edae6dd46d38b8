// query_h1.cu -- the HIBF query kernels for hierarchies with 1 hash function(s): every tuning variant and the
// learned scheduler's feature kernel.
// One translation unit per hash function count keeps the instantiations compiling in parallel.
#include "query.cuh"

namespace hibf_gb300
{
query_kernel_t query_kernel_h1(int v)
{
    return query_kernel_variant<1>(v);
}
query_kernel_t query_block_kernel_h1()
{
    return k_query_blk<1>;
}
features_kernel_t features_kernel_h1()
{
    return k_query_features<1>;
}
} // namespace hibf_gb300
