// Sampling for a decoder: the host side of gfs_sample_for_decoder (include/stim_gb300.h).
//
// Replaces the sampling half of sinter's _CompiledStimThenDecodeSampler.sample
// (glue/sample/src/sinter/_decoding/_stim_then_decode_sampler.py:170-190): detection events bit-packed with
// separate observables (:171-175), the detection-event count (:178-181) and the postselection mask (:183-190).
// Per chunk of shots: the frame and transpose kernels write dense shot-major rows into device buffers,
// feed_popcount_kernel counts their set bits, and with a mask feed_flags / feed_scan / feed_compact drop the
// postselected shots and pack the kept rows in shot order; only the kept rows are copied to the host, on the
// copy stream while the next chunk is sampled into the other slot.
#include "sampler.h"

using namespace gfs_rt;

namespace {

uint64_t up256(uint64_t n) {
    return (n + 255) / 256 * 256;
}

void sample_for_decoder(gfs_sampler *s, uint64_t shots, const uint8_t *mask, uint8_t *dets, uint64_t dstride,
                        uint8_t *obs, uint64_t ostride, uint64_t *out3) {
    if (s->mode != GFS_MODE_DETECTIONS) {
        throw std::invalid_argument("sampler was not created in detection mode");
    }
    const uint64_t D = s->prog.num_detectors, O = s->prog.num_observables;
    const uint64_t drow = (D + 7) / 8, orow = (O + 7) / 8;
    if ((dets && dstride < drow) || (obs && ostride < orow)) {
        throw std::invalid_argument("output row stride too small");
    }
    // The mask as (byte, bits) pairs over its nonzero bytes; bits past the last detector are ignored.
    std::vector<uint32_t> idx;
    std::vector<uint8_t> bits;
    if (mask) {
        for (uint64_t j = 0; j < drow; j++) {
            uint32_t m = mask[j];
            if (j + 1 == drow && (D & 7)) {
                m &= (1u << (D & 7)) - 1;
            }
            if (m) {
                idx.push_back((uint32_t)j);
                bits.push_back((uint8_t)m);
            }
        }
    }
    const uint32_t nmask = (uint32_t)idx.size();
    ck(cudaSetDevice(s->device), "cudaSetDevice");
    // Chunks of whole resident waves of the frame kernel (a partial wave costs nearly a full one), at most
    // about 512 MiB of rows per slot (twice that with a mask: rows plus kept rows), and a multiple of 128 shots so
    // that consecutive chunks continue the stream exactly.
    const uint64_t per_shot = std::max<uint64_t>(1, drow + orow);
    const uint64_t wave = std::max<uint64_t>(128, (uint64_t)s->shape.grid * (uint64_t)s->shape.blocks_per_cta * 128);
    uint64_t chunk = std::max<uint64_t>(1, ((uint64_t)512 << 20) / per_shot / wave) * wave;
    chunk = std::min<uint64_t>(chunk, (shots + 127) / 128 * 128);
    chunk = std::max<uint64_t>(chunk, 128);
    const uint64_t groups = (chunk + gfs::kFeedGroup - 1) / gfs::kFeedGroup;
    const uint64_t dbytes = up256(chunk * drow), obytes = up256(chunk * orow);
    const uint64_t aux_counts = 0, aux_groups = 256, aux_keep = aux_groups + up256(4 * groups),
                   aux_idx = aux_keep + up256(chunk), aux_bits = aux_idx + up256(4 * (uint64_t)nmask),
                   aux_dst = aux_bits + up256(nmask), aux_total = aux_dst + up256(4 * chunk);
    gfs::FeedArgs args[2];
    for (int k = 0; k < 2; k++) {
        s->feed_rows[k].ensure(std::max<uint64_t>(256, dbytes + obytes), s->device);
        if (nmask) {
            s->feed_compact[k].ensure(std::max<uint64_t>(256, dbytes + obytes), s->device);
        }
        s->feed_aux[k].ensure(aux_total, s->device);
        uint8_t *aux = (uint8_t *)s->feed_aux[k].p;
        uint8_t *rows = (uint8_t *)s->feed_rows[k].p;
        uint8_t *crows = nmask ? (uint8_t *)s->feed_compact[k].p : nullptr;
        if (nmask) {
            ck(cudaMemcpyAsync(aux + aux_idx, idx.data(), 4 * (uint64_t)nmask, cudaMemcpyHostToDevice, s->stream),
               "mask upload");
            ck(cudaMemcpyAsync(aux + aux_bits, bits.data(), nmask, cudaMemcpyHostToDevice, s->stream), "mask upload");
        }
        gfs::FeedArgs &a = args[k];
        a = gfs::FeedArgs{};
        a.dets = rows;
        a.obs = rows + dbytes;
        a.drow = drow;
        a.orow = orow;
        a.mask_idx = (const uint32_t *)(aux + aux_idx);
        a.mask_bits = aux + aux_bits;
        a.nmask = nmask;
        a.group_kept = (uint32_t *)(aux + aux_groups);
        a.keep = aux + aux_keep;
        a.counts = (unsigned long long *)(aux + aux_counts);
        a.cdets = crows;
        a.cobs = crows ? crows + dbytes : nullptr;
        a.dst = (uint32_t *)(aux + aux_dst);
    }
    ck(cudaStreamSynchronize(s->stream), "mask upload");
    // Two slots: chunk n samples into slot n % 2 while the kept rows of chunk n - 1 leave on the copy stream (with
    // page-locked destinations the copy overlaps the next chunk's kernels).  The per-chunk counts reach the host
    // through mapped memory (launch_publish_words), not a copy that would queue behind the rows on the copy
    // engine.  A slot is reused once its copy has ended.
    uint64_t kept_total = 0, dropped = 0, events = 0;
    bool copying[2] = {false, false};
    uint64_t n = 0;
    for (uint64_t done = 0; done < shots; n++) {
        const int k = (int)(n & 1);
        gfs::FeedArgs &a = args[k];
        if (copying[k]) {
            ck(cudaEventSynchronize(s->pev[k][3]), "feed copy");
            copying[k] = false;
        }
        const uint64_t cs = std::min<uint64_t>(shots - done, chunk);
        // detections() leaves the rows written and s->stream idle.
        s->detections(cs, GFS_BIT_PACKED, drow ? (uint8_t *)a.dets : nullptr, drow,
                      orow ? (uint8_t *)a.obs : nullptr, orow, true);
        a.nshots = cs;
        ck(cudaMemsetAsync(a.counts, 0, 16, s->stream), "memset");
        ck(gfs::launch_feed_popcount(a, s->stream), "popcount launch");
        if (nmask) {
            ck(gfs::launch_feed_flags(a, s->stream), "flags launch");
            ck(gfs::launch_feed_scan(a, s->stream), "scan launch");
            ck(gfs::launch_feed_compact(a, s->stream), "compact launch");
        }
        ck(gfs::launch_publish_words((const uint32_t *)a.counts, s->h_words_dev + 4, 4, s->stream), "counts publish");
        ck(cudaStreamSynchronize(s->stream), "feed");
        const volatile uint32_t *w = s->h_words + 4;
        const uint64_t ev = (uint64_t)w[0] | ((uint64_t)w[1] << 32), dr = (uint64_t)w[2] | ((uint64_t)w[3] << 32);
        const uint64_t kept = cs - dr;
        dropped += dr;
        events += ev;
        const uint8_t *src = nmask ? a.cdets : a.dets;
        const uint8_t *osrc = nmask ? a.cobs : a.obs;
        if (dets && drow && kept) {
            s->copy_rows(dets + kept_total * dstride, dstride, src, drow, drow, kept, "copy dets");
        }
        if (obs && orow && kept) {
            s->copy_rows(obs + kept_total * ostride, ostride, osrc, orow, orow, kept, "copy obs");
        }
        ck(cudaEventRecord(s->pev[k][3], s->copy_stream), "event");
        copying[k] = true;
        kept_total += kept;
        done += cs;
    }
    ck(cudaStreamSynchronize(s->copy_stream), "copy");
    out3[0] = kept_total;
    out3[1] = dropped;
    out3[2] = events;
}

}  // namespace

extern "C" {

gfs_status gfs_sample_for_decoder(gfs_sampler *s, uint64_t shots, const uint8_t *postselection_mask, uint8_t *dets,
                                  uint64_t dets_stride, uint8_t *obs, uint64_t obs_stride, uint64_t *out3) {
    return guarded([&] {
        sample_for_decoder(s, shots, postselection_mask, dets, dets_stride, obs, obs_stride, out3);
    });
}

}  // extern "C"
