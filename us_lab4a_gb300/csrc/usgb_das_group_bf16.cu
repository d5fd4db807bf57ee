// Receiver-group delay-and-sum kernels for BF16 signal tensors (usgb_das_group.cuh).
#include "usgb_das_group.cuh"

namespace usgb {

cudaError_t launch_das_group_bf16(const DasParams& p, int cf, bool analytic, cudaStream_t stream)
{
	return launch_das_group_storage<STORE_BF16>(p, cf, analytic, stream);
}

cudaError_t launch_das_group_batch_bf16(const BatchDasFrame* frames, const BatchHeader* hdr, const BatchDasConfig& c,
		bool analytic, cudaStream_t stream)
{
	return launch_das_group_batch_storage<STORE_BF16>(frames, hdr, c, analytic, stream);
}

}  // namespace usgb
