/*
 * jn_noalloc.cu — the Hamiltonian product for callers that must not
 * allocate device memory.
 *
 * jn_matvec_device() keeps its scratch (the 64-bit fixed-point accumulator,
 * the FP32 copy of x and two control words) in buffers that jn_open_files()
 * allocates.  Some callers of the product cannot let a library allocate
 * behind their back: a Lanczos driver that has sized its Krylov basis to the
 * device memory it was granted, an application that runs under a fixed
 * memory budget (the reference's max_memory_load), or a solver loop that
 * cannot afford the device-wide synchronisation a cudaMalloc may bring.
 * jn_matvec_device_noalloc() computes the block-tile engine's product (bit
 * for bit what jn_matvec_device gives when the context runs engine 3) with
 * its scratch in a file-scope device array of fixed size instead.  It never
 * calls cudaMalloc, cudaFree or an allocating library routine.
 *
 * The array lives in the library's device image: every GPU that loads the
 * library holds it (JN_NOALLOC_MAX_DIM * 12 + 8 bytes, about 3 MiB) until the
 * process exits.  All calls share it, so calls whose kernels overlap on the
 * GPU (on different streams or from different threads) race and give wrong
 * results; serialise them.  Each call clears the parts that must start at
 * zero before it uses them.
 *
 * Host code cannot use the array's name as a device address (it names a
 * host-side stand-in), so the first call on each device looks the address up
 * with cudaGetSymbolAddress while that device is current and caches it.  That
 * first call should therefore come before any stream capture.  The cache
 * lasts as long as the process: after cudaDeviceReset the cached address is
 * stale, so the entry point must not be called on a device that was reset.
 */
#include <pthread.h>

#include "jn_internal.h"

/* accumulator (8 B), FP32 x (4 B) per basis state, then two control words */
static __device__ __align__(256) unsigned char g_noalloc_scratch[(size_t)JN_NOALLOC_MAX_DIM * 12 + 256];

#define JN_MAX_DEVICES 64
static void *g_scratch_addr[JN_MAX_DEVICES];
static pthread_mutex_t g_scratch_lock = PTHREAD_MUTEX_INITIALIZER;

static jn_status scratch_address(int device, unsigned char **out)
{
	if (device < 0 || device >= JN_MAX_DEVICES) return jn_fail(JN_ERR_INVALID, "device ordinal %d out of range", device);
	pthread_mutex_lock(&g_scratch_lock);
	void *p = g_scratch_addr[device];
	cudaError_t e = cudaSuccess;
	if (!p) {
		e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
		if (e == cudaSuccess) g_scratch_addr[device] = p;
	}
	pthread_mutex_unlock(&g_scratch_lock);
	if (e != cudaSuccess)
		return jn_fail(JN_ERR_CUDA, "cudaGetSymbolAddress(scratch) failed: %s", cudaGetErrorString(e));
	*out = (unsigned char *)p;
	return JN_OK;
}

extern "C" jn_status jn_matvec_device_noalloc(jn_ctx *c, const double *d_x, double *d_y, int accumulate, void *stream)
{
	if (!c || !d_x || !d_y) return jn_fail(JN_ERR_INVALID, "null argument");
	if (d_x == d_y) return jn_fail(JN_ERR_INVALID, "x and y must not alias");
	if (c->plan.btiles_off) return jn_fail(JN_ERR_INVALID, "no block-tile engine: %s", c->plan.btiles_why);
	const int64_t D = c->plan.dim;
	if (D > JN_NOALLOC_MAX_DIM)
		return jn_fail(JN_ERR_INVALID,
			       "dimension %lld exceeds the %d basis states the allocation-free product supports",
			       (long long)D, JN_NOALLOC_MAX_DIM);
	if (c->precision == 32 && !c->d_me32)
		return jn_fail(JN_ERR_INVALID, "FP32 matrix elements are not set up: call jn_set_precision first");
	int dev = 0;
	cudaError_t e = cudaGetDevice(&dev);
	if (e != cudaSuccess) return jn_fail(JN_ERR_CUDA, "cudaGetDevice failed: %s", cudaGetErrorString(e));
	if (dev != c->device)
		return jn_fail(JN_ERR_INVALID, "the current device (%d) is not the context's device (%d)", dev, c->device);
	unsigned char *base = NULL;
	jn_status s = scratch_address(dev, &base);
	if (s) return s;
	unsigned long long *acc = (unsigned long long *)base;
	float *x32 = (float *)(base + (size_t)JN_NOALLOC_MAX_DIM * 8);
	unsigned int *ctrl = (unsigned int *)(base + (size_t)JN_NOALLOC_MAX_DIM * 12);
	return jn_enqueue_tiles(c, d_x, d_y, accumulate, stream ? (cudaStream_t)stream : c->stream, NULL, NULL, acc, ctrl,
				x32, 1);
}
