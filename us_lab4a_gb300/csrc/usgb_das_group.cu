// Receiver-group delay-and-sum: dispatch by storage type to the kernels of
// usgb_das_group.cuh, instantiated in usgb_das_group_{f32,f16,bf16}.cu.
#include "usgb_das_group.cuh"

namespace usgb {

cudaError_t launch_das_group_f32(const DasParams& p, int cf, bool analytic, cudaStream_t stream);
cudaError_t launch_das_group_f16(const DasParams& p, int cf, bool analytic, cudaStream_t stream);
cudaError_t launch_das_group_bf16(const DasParams& p, int cf, bool analytic, cudaStream_t stream);
cudaError_t launch_das_group_batch_f32(const BatchDasFrame*, const BatchHeader*, const BatchDasConfig&, bool, cudaStream_t);
cudaError_t launch_das_group_batch_f16(const BatchDasFrame*, const BatchHeader*, const BatchDasConfig&, bool, cudaStream_t);
cudaError_t launch_das_group_batch_bf16(const BatchDasFrame*, const BatchHeader*, const BatchDasConfig&, bool, cudaStream_t);

cudaError_t launch_das_group_batch(const BatchDasFrame* frames, const BatchHeader* hdr, const BatchDasConfig& c,
		int storage, bool analytic, cudaStream_t stream)
{
	switch (storage) {
	case STORE_F16: return launch_das_group_batch_f16(frames, hdr, c, analytic, stream);
	case STORE_BF16: return launch_das_group_batch_bf16(frames, hdr, c, analytic, stream);
	default: return launch_das_group_batch_f32(frames, hdr, c, analytic, stream);
	}
}

size_t das_group_smem_bytes(unsigned numTx, unsigned numRx, unsigned tileCols, unsigned tileRows, unsigned capBytes,
		unsigned stages)
{
	return group_layout_bytes(numTx, numRx, tileCols, tileRows, capBytes, stages);
}

cudaError_t launch_das_group(const DasParams& p, int storage, int cf, bool analytic, cudaStream_t stream)
{
	switch (storage) {
	case STORE_F16: return launch_das_group_f16(p, cf, analytic, stream);
	case STORE_BF16: return launch_das_group_bf16(p, cf, analytic, stream);
	default: return launch_das_group_f32(p, cf, analytic, stream);
	}
}

}  // namespace usgb
