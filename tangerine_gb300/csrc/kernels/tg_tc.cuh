// Fifth-generation tensor core (tcgen05) building blocks for sm_103a, written as inline
// PTX: tensor-memory allocation, BF16 x BF16 -> FP32 matrix multiply-accumulate with
// operands in shared memory and the accumulator in tensor memory, completion through an
// mbarrier, tensor-memory loads, and bulk global -> shared copies.
//
// Shared-memory operands use the no-swizzle canonical layout.  A "core matrix" is 8 rows
// of 16 bytes (8 x 8 bf16) stored contiguously (128 bytes).  For a row-major tile of R
// rows by C bf16 columns (both multiples of 8) this build stores element (r, c) at byte
//     (r / 8) * (C / 8) * 128 + (c / 8) * 128 + (r % 8) * 16 + (c % 8) * 2.
// Read with K = columns ("K-major": rows are M or N) the descriptor's leading byte offset
// (core-matrix step along K) is 128 and its stride byte offset (step along M/N) is
// (C / 8) * 128.  Read with K = rows ("MN-major": columns are M or N) the same bytes
// describe the transposed tile with the two offsets exchanged: the step along M/N is 128
// (the stride byte offset) and the step along K is (C / 8) * 128 (the leading byte
// offset).  One buffer therefore serves as X (samples x features, K = features) and as
// X^T (features x samples, K = samples) without a transposed copy.
//
// Every wait is bounded by the global timer; a wait that runs out reports failure and the
// caller records an error status instead of spinning forever.
#pragma once

#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace tg
{
	namespace tc
	{
		constexpr uint64_t kWaitLimitNs = 2000000000ull;     // 2 s

		__device__ __forceinline__ uint32_t SmemAddr(const void* p)
		{
			return static_cast<uint32_t>(__cvta_generic_to_shared(p));
		}

		__device__ __forceinline__ uint64_t GlobalTimer()
		{
			uint64_t t;
			asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
			return t;
		}

		// Byte offset of element (r, c) of a row-major R x C bf16 tile in the core-matrix
		// layout above (C = the tile's column count).
		__host__ __device__ __forceinline__ uint32_t TileOffset(uint32_t r, uint32_t c, uint32_t C)
		{
			return (r >> 3) * (C >> 3) * 128u + (c >> 3) * 128u + (r & 7u) * 16u + (c & 7u) * 2u;
		}

		// Shared-memory matrix descriptor, no swizzle: start address, leading byte offset
		// (core-matrix step along K), stride byte offset (step along M/N), all >> 4, and
		// the descriptor version bits (46-47 = 1) tcgen05 expects.
		__device__ __forceinline__ uint64_t Descriptor(uint32_t addr, uint32_t lbo, uint32_t sbo)
		{
			uint64_t d = 0;
			d |= static_cast<uint64_t>((addr >> 4) & 0x3FFFu);
			d |= static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16;
			d |= static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32;
			d |= static_cast<uint64_t>(1) << 46;
			return d;
		}

		// Descriptor of a tile read K-major (K along its columns), starting at column c0.
		__device__ __forceinline__ uint64_t KMajor(const void* tile, uint32_t C, uint32_t c0 = 0)
		{
			return Descriptor(SmemAddr(tile) + (c0 >> 3) * 128u, 128u, (C >> 3) * 128u);
		}

		// Descriptor of a tile read MN-major (K along its rows), starting at row r0 and
		// column c0 (r0 a multiple of 8).
		__device__ __forceinline__ uint64_t MNMajor(const void* tile, uint32_t C, uint32_t r0 = 0, uint32_t c0 = 0)
		{
			return Descriptor(SmemAddr(tile) + (r0 >> 3) * (C >> 3) * 128u + (c0 >> 3) * 128u, (C >> 3) * 128u, 128u);
		}

		// Instruction descriptor of kind::f16 with BF16 A and B and an FP32 accumulator.
		// Bits: 4-5 accumulator format (1 = F32), 7-9 A format (1 = BF16), 10-12 B format,
		// 15 A major (1 = MN), 16 B major, 17-22 N >> 3, 24-28 M >> 4.
		__host__ __device__ constexpr uint32_t InstrBf16(int M, int N, bool a_mn, bool b_mn)
		{
			return (1u << 4) | (1u << 7) | (1u << 10) | ((a_mn ? 1u : 0u) << 15) | ((b_mn ? 1u : 0u) << 16) |
				(static_cast<uint32_t>(N >> 3) << 17) | (static_cast<uint32_t>(M >> 4) << 24);
		}

		// D[tmem] (+)= A * B^T for one K = 16 step; issued by a single thread.
		__device__ __forceinline__ void Mma(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate)
		{
			asm volatile(
				"{\n"
				".reg .pred p;\n"
				"setp.ne.b32 p, %4, 0;\n"
				"tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
				"}\n"
				:: "r"(tmem_d), "l"(a), "l"(b), "r"(idesc), "r"(accumulate) : "memory");
		}

		// Arrives once on `bar` when every tcgen05.mma this thread issued so far completes.
		__device__ __forceinline__ void Commit(uint64_t* bar)
		{
			asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
				:: "r"(SmemAddr(bar)) : "memory");
		}

		__device__ __forceinline__ void FenceBeforeSync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
		__device__ __forceinline__ void FenceAfterSync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
		// Makes this thread's ordinary shared-memory stores visible to the tensor core.
		__device__ __forceinline__ void FenceProxyAsync() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

		// Tensor-memory allocation by one whole warp; the base address lands in *slot.
		__device__ __forceinline__ void Alloc(uint32_t* slot, uint32_t columns)
		{
			asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
				:: "r"(SmemAddr(slot)), "r"(columns) : "memory");
			asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
		}

		__device__ __forceinline__ void Dealloc(uint32_t base, uint32_t columns)
		{
			asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(base), "r"(columns) : "memory");
		}

		__device__ __forceinline__ void BarInit(uint64_t* bar, uint32_t count)
		{
			asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(SmemAddr(bar)), "r"(count) : "memory");
			asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
		}

		__device__ __forceinline__ bool BarTryWait(uint64_t* bar, uint32_t parity)
		{
			uint32_t ok;
			asm volatile(
				"{\n"
				".reg .pred p;\n"
				"mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
				"selp.u32 %0, 1, 0, p;\n"
				"}\n"
				: "=r"(ok) : "r"(SmemAddr(bar)), "r"(parity) : "memory");
			return ok != 0;
		}

		// Waits for the phase with this parity to complete; false after `limit_ns`.
		__device__ __forceinline__ bool BarWaitFor(uint64_t* bar, uint32_t parity, uint64_t limit_ns)
		{
			if (BarTryWait(bar, parity)) return true;
			const uint64_t t0 = GlobalTimer();
			while (!BarTryWait(bar, parity))
				if (GlobalTimer() - t0 > limit_ns) return false;
			return true;
		}

		// BarWaitFor with the library's limit.
		__device__ __forceinline__ bool BarWait(uint64_t* bar, uint32_t parity)
		{
			return BarWaitFor(bar, parity, kWaitLimitNs);
		}

		// Bulk copy of `bytes` (multiple of 16, both addresses 16-byte aligned) from global
		// to shared memory, completing a transaction count on `bar` (one arrival).
		__device__ __forceinline__ void BulkLoad(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
		{
			asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(SmemAddr(bar)), "r"(bytes) : "memory");
			asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
				:: "r"(SmemAddr(dst)), "l"(src), "r"(bytes), "r"(SmemAddr(bar)) : "memory");
		}

		// 16 consecutive FP32 columns of this thread's tensor-memory lane (32x32b shape:
		// warp w of the CTA reads lanes 32w .. 32w + 31, thread t lane 32w + t).
		__device__ __forceinline__ void Load16(uint32_t taddr, float (&v)[16])
		{
			uint32_t r[16];
			asm volatile(
				"tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
				: "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
				  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
				: "r"(taddr) : "memory");
			asm volatile("tcgen05.wait::ld.sync.aligned;"
				: "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
				  "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15])
				:: "memory");
#pragma unroll
			for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
		}

		// Tensor-memory address of (lane, column) relative to an allocation base.
		__device__ __forceinline__ uint32_t TmemAddr(uint32_t base, uint32_t lane, uint32_t column)
		{
			return base + (lane << 16) + column;
		}

		// Stores 8 consecutive bf16 values (columns c .. c + 7, c a multiple of 8) of row r.
		__device__ __forceinline__ void StoreRow8(void* tile, uint32_t r, uint32_t c, uint32_t C, const float (&v)[8])
		{
			__nv_bfloat162 p[4];
#pragma unroll
			for (int i = 0; i < 4; ++i) p[i] = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
			*reinterpret_cast<uint4*>(static_cast<char*>(tile) + TileOffset(r, c, C)) = *reinterpret_cast<const uint4*>(p);
		}
	}
}
