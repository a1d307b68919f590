/*
 * orc.h - C interface of the CPU oracles of the radar chain.
 *
 * TEST INFRASTRUCTURE ONLY. Two libraries implement this interface:
 *
 *   oracle/_build/liborc.so     orc_port.c: a plain-C restatement of the
 *                               reference model's algorithms (builds anywhere);
 *   oracle/_ref/liborc_ref.so   ref_chain.cpp: a composition driver over the
 *                               reference's own model/cpp headers (builds only
 *                               where the reference sources are present).
 *
 * Only tests, the smoke check and the CPU-baseline leg of the benchmark load
 * either library, and only to check or time against the CUDA product. The
 * structures are the product's own (include/rd_chain.h), so outputs compare
 * field for field.
 */
#ifndef ORC_H_
#define ORC_H_

#include <stdint.h>

#include "../include/rd_chain.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_chain orc_chain;

/* Chain composition in the order of rtl/top/benchmark_sim_top.sv. */
int orc_chain_create(const rd_config* cfg, const rd_cplx16* coeff,
                     const rd_cplx16* weights, const uint32_t* pair_x,
                     const uint32_t* pair_y, uint32_t n_pairs,
                     orc_chain** out);
void orc_chain_destroy(orc_chain* ch);
int orc_chain_set_coeff(orc_chain* ch, const rd_cplx16* coeff);
int orc_chain_set_weights(orc_chain* ch, const rd_cplx16* w);
/* n samples per channel from [n_chan][ld]; threads > 1 fans out over
 * independent units (channels, bins, beams). */
int orc_chain_process(orc_chain* ch, const rd_cplx16* adc, uint64_t n,
                      uint64_t ld, rd_output* out, int threads);
int orc_chain_flush_cov(orc_chain* ch, rd_output* out);
int orc_chain_stats(const orc_chain* ch, rd_stats* st);
int orc_chain_read_history(orc_chain* ch, uint32_t bin, uint32_t frame_off,
                           rd_cplx16* vec, uint32_t* frame_id, uint32_t* flags);
int orc_chain_set_history_depth(orc_chain* ch, uint32_t frames);

/* Per-block oracles, same meaning as the rd_* entry points of rd_chain.h. */
int orc_pfb_run(uint32_t phases, uint32_t taps, const rd_cplx16* coeff,
                rd_cplx16* state, const rd_cplx16* in, uint32_t beats,
                rd_cplx16* out, uint8_t* flags_out);
int orc_fft_run(uint32_t n_fft, uint32_t spc, uint32_t scale_sched, int reorder,
                const rd_cplx16* in, uint32_t frames, rd_cplx16* out,
                rd_cplx16* bins, uint8_t* stage_flags);
int orc_bf_run(uint32_t n_ant, uint32_t n_beams, const rd_cplx16* w,
               const rd_cplx16* x, uint64_t n_vec, rd_cplx16* y, int64_t* acc,
               uint8_t* flags);
int orc_power_run(const rd_cplx16* x, uint64_t n, int64_t* power);
int orc_cross_power_run(const rd_cplx16* x, const rd_cplx16* y, uint64_t n,
                        int64_t* cross);
int orc_cfar_run(const int64_t* cells, uint32_t n, uint32_t frames,
                 const rd_config* cfg, const uint32_t* frame_ids,
                 rd_event* events, uint64_t cap, uint64_t* n_events);
int orc_packetize(const rd_event* ev, uint64_t n, uint32_t packet_w,
                  uint32_t src_id, uint32_t dest, uint32_t vc, uint32_t seq0,
                  uint32_t* flits);
int orc_fxp_apply(const uint32_t* op, const int64_t* a, const int64_t* b,
                  const uint32_t* sh, const uint32_t* w, uint64_t n, int64_t* y,
                  uint8_t* flags);
/* The 1024-entry Q1.15 twiddle table (fft_twiddle_table.hpp:43). */
/* liborc_ref.so only: the reference's packet_model::Scoreboard (see
 * ref_chain.cpp) */
int orc_ref_scoreboard(uint32_t packet_w, uint32_t radix, uint32_t stages,
                       const uint32_t* inj, uint64_t n_inj_flits, const uint32_t* obs_port,
                       const uint32_t* obs, uint64_t n_obs, uint64_t* counts, char* log,
                       uint64_t log_cap);

void orc_twiddles(uint32_t* out1024);
const char* orc_name(void);

#ifdef __cplusplus
}
#endif

#endif /* ORC_H_ */
