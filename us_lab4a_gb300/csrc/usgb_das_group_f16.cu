// Receiver-group delay-and-sum kernels for F16 signal tensors (usgb_das_group.cuh).
#include "usgb_das_group.cuh"

namespace usgb {

cudaError_t launch_das_group_f16(const DasParams& p, int cf, bool analytic, cudaStream_t stream)
{
	return launch_das_group_storage<STORE_F16>(p, cf, analytic, stream);
}

cudaError_t launch_das_group_batch_f16(const BatchDasFrame* frames, const BatchHeader* hdr, const BatchDasConfig& c,
		bool analytic, cudaStream_t stream)
{
	return launch_das_group_batch_storage<STORE_F16>(frames, hdr, c, analytic, stream);
}

}  // namespace usgb
