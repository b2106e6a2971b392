/*
 * Genotype record writers of convertf on the device: the resident panel (gp_load_genotypes,
 * packed 2-bit code, MSB first, 3 = missing) re-encoded for a list of output SNPs and an
 * ordered list of output samples, in the record layout of one output format:
 *
 *   GP_OUT_PACKEDANCESTRYMAP  outpack (src/mcio.c:2343-2457): max(ceil(n/4), 48) bytes per
 *                             SNP, sample j at byte j>>2, bits (3-(j&3))*2, value = count of
 *                             the first allele, 3 = missing, unused bits 0 (wbuff on a zeroed
 *                             buffer, :2429-2437)
 *   GP_OUT_PACKEDPED          outpackped (:3619-3703) + setbedbuff (:3706-3724) + bedval
 *                             (:3727-3741): ceil(n/4) bytes, sample j at bits (j&3)*2 (LSB
 *                             first); g -> 2-g then 0 -> 00, 1 -> 10, 2 -> 11, missing 01;
 *                             unused bits 10 (the buffer starts as 0xAA)
 *   GP_OUT_EIGENSTRAT         outeigenstrat (:3262-3320): n characters '0' '1' '2' or '9'
 *                             (missing), then '\n'
 *
 * A flipped SNP (flip1, src/convertf.c:1017-1026: flipalleles, src/admutils.c:204-215) has
 * every observed g replaced by 2 - g before encoding.
 *
 * The work is byte-level and HBM-bound (one read of each selected record, one write of each
 * output record).  k_encode_tile stages groups of records in shared memory so that global
 * stores are 16 bytes wide; identity sample lists transform whole 32-bit words (the four
 * samples of an output byte are the four codes of one input byte).  k_encode (one warp per
 * record, byte stores) serves records too large for shared memory.
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "gp_internal.h"

/* one packed input code (0, 1, 2 or 3 = missing) after the optional flip */
__device__ __forceinline__ unsigned flip_code(unsigned c, bool flip)
{
  return (flip && c < 3u) ? 2u - c : c;
}

/* bed code of a packed code (setbedbuff/bedval after g -> 2-g) */
__device__ __forceinline__ unsigned bed_code(unsigned c)
{
  /* g = 0 -> 2-g = 2 -> 11; g = 1 -> 10; g = 2 -> 00; missing -> 01 */
  return c == 0u ? 3u : (c == 1u ? 2u : (c == 2u ? 0u : 1u));
}

/* code of output sample k of record rec (k < n); idx == NULL: sample k itself */
__device__ __forceinline__ unsigned sample_code(const uint8_t *rec, const int32_t *idx, int32_t k)
{
  const int32_t s = idx ? __ldg(idx + k) : k;
  return (rec[s >> 2] >> ((3 - (s & 3)) * 2)) & 3u;
}

template <int FMT>
__global__ void k_encode(const uint8_t *__restrict__ geno, int64_t rlen_dev,
                         const int32_t *__restrict__ idx, int32_t n,
                         const int64_t *__restrict__ snps, const uint8_t *__restrict__ flips,
                         int64_t nrec, int64_t out_rb, uint8_t *__restrict__ out)
{
  const int lane = threadIdx.x & 31;
  const int64_t warp0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int32_t nfull = n >> 2; /* output bytes holding four samples */
  for (int64_t r = warp0; r < nrec; r += nwarps) {
    const uint8_t *rec = geno + snps[r] * rlen_dev;
    const bool flip = flips != NULL && flips[r] != 0;
    uint8_t *o = out + r * out_rb;
    if (FMT == GP_OUT_EIGENSTRAT) {
      /* four characters per lane per round */
      for (int64_t c0 = (int64_t)lane * 4; c0 < out_rb; c0 += 128) {
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          const int64_t c = c0 + t;
          if (c < n) {
            const unsigned g = flip_code(sample_code(rec, idx, (int32_t)c), flip);
            o[c] = g < 3u ? (uint8_t)('0' + g) : (uint8_t)'9';
          } else if (c == n) {
            o[c] = '\n';
          }
        }
      }
    } else {
      for (int64_t b0 = (int64_t)lane * 4; b0 < out_rb; b0 += 128) {
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          const int64_t b = b0 + t;
          if (b >= out_rb) break;
          unsigned byte;
          if (b < nfull || (b == nfull && (n & 3))) {
            const int nin = b < nfull ? 4 : (n & 3);
            unsigned code[4];
            if (idx == NULL) {
              const unsigned v = rec[b];
#pragma unroll
              for (int u = 0; u < 4; ++u) code[u] = (v >> ((3 - u) * 2)) & 3u;
            } else {
#pragma unroll
              for (int u = 0; u < 4; ++u)
                code[u] = u < nin ? sample_code(rec, idx, (int32_t)(4 * b + u)) : 0u;
            }
            byte = 0u;
#pragma unroll
            for (int u = 0; u < 4; ++u) {
              if (FMT == GP_OUT_PACKEDANCESTRYMAP)
                byte |= (u < nin ? flip_code(code[u], flip) : 0u) << ((3 - u) * 2);
              else
                byte |= (u < nin ? bed_code(flip_code(code[u], flip)) : 2u) << (u * 2);
            }
          } else {
            byte = FMT == GP_OUT_PACKEDANCESTRYMAP ? 0u : 0xAAu;
          }
          o[b] = (uint8_t)byte;
        }
      }
    }
  }
}

/* g -> 2 - g on the 16 codes of a word (00 <-> 10; 01 and 11 unchanged): toggle the high bit
 * of every code whose low bit is 0 */
__device__ __forceinline__ uint32_t flip_word(uint32_t w)
{
  return w ^ ((~w & 0x55555555u) << 1);
}

/* four packed bytes -> four bed bytes: each code (h, l) becomes (~h, ~(h ^ l)) (0 -> 11,
 * 1 -> 10, 2 -> 00, 3 -> 01), then the four codes of each byte are reversed (MSB-first to
 * LSB-first sample order) */
__device__ __forceinline__ uint32_t bed_word(uint32_t w)
{
  const uint32_t h = w & 0xAAAAAAAAu, l = w & 0x55555555u;
  uint32_t x = (~h & 0xAAAAAAAAu) | (~((h >> 1) ^ l) & 0x55555555u);
  x = ((x & 0x0F0F0F0Fu) << 4) | ((x >> 4) & 0x0F0F0F0Fu);
  return ((x & 0x33333333u) << 2) | ((x >> 2) & 0x33333333u);
}

/*
 * Tiled form of k_encode: a block encodes R consecutive output records into shared memory
 * (identity sample lists read each input record with 16-byte loads and transform whole words;
 * sample subsets gather per sample), then writes the group's flat byte range with 16-byte
 * stores (bytes at the two unaligned ends).  Shared memory is offset so that it has the
 * alignment of the global destination.
 */
template <int FMT>
__global__ void __launch_bounds__(256) k_encode_tile(
    const uint8_t *__restrict__ geno, int64_t rlen_dev, const int32_t *__restrict__ idx,
    int32_t n, const int64_t *__restrict__ snps, const uint8_t *__restrict__ flips, int64_t nrec,
    int64_t out_rb, uint8_t *__restrict__ out, int32_t R)
{
  extern __shared__ __align__(16) uint8_t sm[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  const int32_t nb_in = (n + 3) >> 2;   /* input bytes holding the n samples */
  const int rem = n & 3;                /* samples in a partial last byte (0: none) */
  for (int64_t g0 = (int64_t)blockIdx.x * R; g0 < nrec; g0 += (int64_t)gridDim.x * R) {
    const int64_t g1 = g0 + R < nrec ? g0 + R : nrec;
    uint8_t *gdst = out + g0 * out_rb;
    const int off = (int)((uintptr_t)gdst & 15);
    for (int64_t r = g0 + warp; r < g1; r += nwarp) {
      uint8_t *so = sm + off + (r - g0) * out_rb;
      const uint8_t *rec = geno + snps[r] * rlen_dev;
      const bool flip = flips != NULL && flips[r] != 0;
      if (idx == NULL) {
        for (int32_t q = lane * 16; q < nb_in; q += 512) {
          const uint4 v = *reinterpret_cast<const uint4 *>(rec + q);
          uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            if (flip) w[i] = flip_word(w[i]);
            if (FMT == GP_OUT_PACKEDPED) w[i] = bed_word(w[i]);
          }
#pragma unroll
          for (int k = 0; k < 16; ++k) {
            const int32_t b = q + k;
            if (b >= nb_in) break;
            uint32_t val = (w[k >> 2] >> (8 * (k & 3))) & 0xFFu;
            if (FMT == GP_OUT_EIGENSTRAT) {
#pragma unroll
              for (int u = 0; u < 4; ++u) {
                const int32_t smp = 4 * b + u;
                if (smp < n) {
                  const uint32_t c = (val >> (6 - 2 * u)) & 3u;
                  so[smp] = (uint8_t)(c < 3u ? '0' + c : '9');
                }
              }
            } else {
              if (rem && b == nb_in - 1) {
                if (FMT == GP_OUT_PACKEDANCESTRYMAP)
                  val &= (0xFFu << (8 - 2 * rem)) & 0xFFu;
                else
                  val = (val & ((1u << (2 * rem)) - 1u)) | (0xAAu & ~((1u << (2 * rem)) - 1u));
              }
              so[b] = (uint8_t)val;
            }
          }
        }
      } else if (FMT == GP_OUT_EIGENSTRAT) {
        for (int32_t c = lane; c < n; c += 32) {
          const unsigned g = flip_code(sample_code(rec, idx, c), flip);
          so[c] = g < 3u ? (uint8_t)('0' + g) : (uint8_t)'9';
        }
      } else {
        for (int32_t b = lane; b < nb_in; b += 32) {
          const int nin = (rem && b == nb_in - 1) ? rem : 4;
          unsigned byte = 0u;
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const unsigned c = u < nin ? flip_code(sample_code(rec, idx, 4 * b + u), flip) : 0u;
            if (FMT == GP_OUT_PACKEDANCESTRYMAP)
              byte |= (u < nin ? c : 0u) << ((3 - u) * 2);
            else
              byte |= (u < nin ? bed_code(c) : 2u) << (u * 2);
          }
          so[b] = (uint8_t)byte;
        }
      }
      /* the rest of the record: packedancestrymap's zero bytes up to 48, EIGENSTRAT's '\n' */
      if (FMT == GP_OUT_EIGENSTRAT) {
        if (lane == 0) so[n] = '\n';
      } else {
        for (int64_t b = nb_in + lane; b < out_rb; b += 32) so[b] = 0;
      }
    }
    __syncthreads();
    /* the group's bytes [0, len) -> gdst: unaligned head and tail by bytes, the rest by 16 */
    const int64_t len = (g1 - g0) * out_rb;
    const int64_t head = ((16 - off) & 15) < len ? ((16 - off) & 15) : len;
    const int64_t nvec = (len - head) >> 4;
    const int64_t tail0 = head + nvec * 16;
    for (int64_t i = threadIdx.x; i < head; i += blockDim.x) gdst[i] = sm[off + i];
    for (int64_t v = threadIdx.x; v < nvec; v += blockDim.x)
      *reinterpret_cast<uint4 *>(gdst + head + 16 * v) =
          *reinterpret_cast<const uint4 *>(sm + off + head + 16 * v);
    for (int64_t i = tail0 + threadIdx.x; i < len; i += blockDim.x) gdst[i] = sm[off + i];
    __syncthreads();
  }
}

extern "C" int64_t gp_record_bytes(int32_t format, int32_t nsamples)
{
  if (nsamples < 0) return -1;
  const int64_t q = ((int64_t)nsamples + 3) / 4;
  switch (format) {
  case GP_OUT_PACKEDANCESTRYMAP:
    return q > 48 ? q : 48;
  case GP_OUT_PACKEDPED:
    return q;
  case GP_OUT_EIGENSTRAT:
    return (int64_t)nsamples + 1;
  default:
    return -1;
  }
}

extern "C" int gp_encode_records(gp_ctx *ctx, int32_t format, const int32_t *sample_index,
                                 int32_t nsamples, const int64_t *snp_index, const uint8_t *flip,
                                 int64_t nsnps, uint8_t *out, int32_t out_on_device)
{
  if (!ctx) return GP_ERR_ARG;
  const int64_t rb = gp_record_bytes(format, nsamples);
  if (rb < 0 || nsnps < 0 || (nsnps > 0 && (!snp_index || !out)))
    return gp_fail(ctx, GP_ERR_ARG, "gp_encode_records: bad format %d, %d samples or %lld SNPs",
                   format, nsamples, (long long)nsnps);
  if (!ctx->d_geno) return gp_fail(ctx, GP_ERR_STATE, "gp_encode_records: no genotypes loaded");
  if (nsnps == 0) return GP_OK;
  /* the sample list: checked on the host (every index inside the panel) */
  bool identity = sample_index == NULL;
  if (sample_index) {
    identity = nsamples <= ctx->nind_all;
    for (int32_t k = 0; k < nsamples; ++k) {
      if (sample_index[k] < 0 || sample_index[k] >= ctx->nind_all)
        return gp_fail(ctx, GP_ERR_ARG, "gp_encode_records: sample %d out of range", sample_index[k]);
      if (sample_index[k] != k) identity = false;
    }
  } else if (nsamples > ctx->nind_all) {
    return gp_fail(ctx, GP_ERR_ARG, "gp_encode_records: %d samples > %d", nsamples, ctx->nind_all);
  }
  for (int64_t i = 0; i < nsnps; ++i)
    if (snp_index[i] < 0 || snp_index[i] >= ctx->nsnp_all)
      return gp_fail(ctx, GP_ERR_ARG, "gp_encode_records: SNP %lld out of range",
                     (long long)snp_index[i]);
  GP_CUDA(ctx, cudaSetDevice(ctx->device));
  /* scratch: sample list, then per chunk the SNP list, flips and (host output) records */
  const int64_t chunk_bytes = (int64_t)64 << 20;
  int64_t chunk = out_on_device ? nsnps : chunk_bytes / rb;
  if (chunk < 1) chunk = 1;
  if (chunk > nsnps) chunk = nsnps;
  const size_t idx_bytes = identity ? 0 : ((sizeof(int32_t) * (size_t)nsamples + 255) & ~(size_t)255);
  const size_t snp_bytes = (sizeof(int64_t) * (size_t)chunk + 255) & ~(size_t)255;
  const size_t flip_bytes = ((size_t)chunk + 255) & ~(size_t)255;
  const size_t rec_bytes = out_on_device ? 0 : (size_t)(chunk * rb);
  uint8_t *base;
  int rc = gp_scratch(ctx, idx_bytes + snp_bytes + flip_bytes + rec_bytes + 256, (void **)&base);
  if (rc) return rc;
  int32_t *d_idx = identity ? NULL : (int32_t *)base;
  int64_t *d_snps = (int64_t *)(base + idx_bytes);
  uint8_t *d_flip = base + idx_bytes + snp_bytes;
  uint8_t *d_rec = base + idx_bytes + snp_bytes + flip_bytes;
  if (!identity)
    GP_CUDA(ctx, gp_memcpy(ctx, d_idx, sample_index, sizeof(int32_t) * (size_t)nsamples,
                           cudaMemcpyHostToDevice, ctx->stream));
  for (int64_t s0 = 0; s0 < nsnps; s0 += chunk) {
    const int64_t nc = nsnps - s0 < chunk ? nsnps - s0 : chunk;
    GP_CUDA(ctx, gp_memcpy(ctx, d_snps, snp_index + s0, sizeof(int64_t) * (size_t)nc,
                           cudaMemcpyHostToDevice, ctx->stream));
    if (flip)
      GP_CUDA(ctx, gp_memcpy(ctx, d_flip, flip + s0, (size_t)nc, cudaMemcpyHostToDevice,
                             ctx->stream));
    uint8_t *dst = out_on_device ? out + s0 * rb : d_rec;
    const int threads = 256;
    const uint8_t *fl = flip ? d_flip : NULL;
    /* tiled kernel: R records (about 32 KB) per block in shared memory */
    int64_t R = ((int64_t)32 << 10) / rb;
    if (R < 1) R = 1;
    if (R > 64) R = 64;
    const size_t smem = (size_t)((16 + R * rb + 16 + 15) & ~(int64_t)15);
    if (out_on_device) GP_CUDA(ctx, cudaEventRecord(ctx->ev_g0, ctx->stream));
    if (smem <= 200 * 1024) {
      int64_t blocks = (nc + R - 1) / R;
      const int64_t cap = (int64_t)ctx->num_sms * 8;
      if (blocks > cap) blocks = cap;
      switch (format) {
      case GP_OUT_PACKEDANCESTRYMAP:
        GP_CUDA(ctx, gp_allow_smem(ctx, (const void *)k_encode_tile<GP_OUT_PACKEDANCESTRYMAP>));
        k_encode_tile<GP_OUT_PACKEDANCESTRYMAP><<<(unsigned)blocks, threads, smem, ctx->stream>>>(
            ctx->d_geno, ctx->rlen_dev, d_idx, nsamples, d_snps, fl, nc, rb, dst, (int32_t)R);
        break;
      case GP_OUT_PACKEDPED:
        GP_CUDA(ctx, gp_allow_smem(ctx, (const void *)k_encode_tile<GP_OUT_PACKEDPED>));
        k_encode_tile<GP_OUT_PACKEDPED><<<(unsigned)blocks, threads, smem, ctx->stream>>>(
            ctx->d_geno, ctx->rlen_dev, d_idx, nsamples, d_snps, fl, nc, rb, dst, (int32_t)R);
        break;
      default:
        GP_CUDA(ctx, gp_allow_smem(ctx, (const void *)k_encode_tile<GP_OUT_EIGENSTRAT>));
        k_encode_tile<GP_OUT_EIGENSTRAT><<<(unsigned)blocks, threads, smem, ctx->stream>>>(
            ctx->d_geno, ctx->rlen_dev, d_idx, nsamples, d_snps, fl, nc, rb, dst, (int32_t)R);
        break;
      }
      GP_LAUNCH_CHECK(ctx, "k_encode_tile");
    } else {
    int64_t blocks = (nc + (threads / 32) - 1) / (threads / 32);
    const int64_t cap = (int64_t)ctx->num_sms * 16;
    if (blocks > cap) blocks = cap;
    switch (format) {
    case GP_OUT_PACKEDANCESTRYMAP:
      k_encode<GP_OUT_PACKEDANCESTRYMAP><<<(unsigned)blocks, threads, 0, ctx->stream>>>(
          ctx->d_geno, ctx->rlen_dev, d_idx, nsamples, d_snps, fl, nc, rb, dst);
      break;
    case GP_OUT_PACKEDPED:
      k_encode<GP_OUT_PACKEDPED><<<(unsigned)blocks, threads, 0, ctx->stream>>>(
          ctx->d_geno, ctx->rlen_dev, d_idx, nsamples, d_snps, fl, nc, rb, dst);
      break;
    default:
      k_encode<GP_OUT_EIGENSTRAT><<<(unsigned)blocks, threads, 0, ctx->stream>>>(
          ctx->d_geno, ctx->rlen_dev, d_idx, nsamples, d_snps, fl, nc, rb, dst);
      break;
    }
    GP_LAUNCH_CHECK(ctx, "k_encode");
    }
    if (out_on_device) GP_CUDA(ctx, cudaEventRecord(ctx->ev_g1, ctx->stream));
    if (!out_on_device)
      GP_CUDA(ctx, gp_memcpy(ctx, out + s0 * rb, d_rec, (size_t)(nc * rb), cudaMemcpyDeviceToHost,
                             ctx->stream));
  }
  GP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (out_on_device) {
    float ms = 0.f;
    GP_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev_g0, ctx->ev_g1));
    ctx->encode_ms = ms;
  }
  return GP_OK;
}

extern "C" int gp_last_encode_time(const gp_ctx *ctx, double *ms)
{
  if (!ctx || !ms) return GP_ERR_ARG;
  *ms = ctx->encode_ms;
  return GP_OK;
}
