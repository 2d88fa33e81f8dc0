// Checkpoint files (host code only): the writer and reader behind
// gb_checkpoint_write / gb_checkpoint_read and the context and batch saves
// and loads. The layout is documented with gb_checkpoint_info in vipp_gb300.h.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>

#include "../../include/vipp_gb300.h"

namespace gb {

// Writes the file under path + ".tmp" and renames it over path. seg_offsets
// may be NULL for one system ({0, n}); m_per_system may be NULL (info->cfg.m
// for every system). Returns a gb_status; err holds the message.
int checkpoint_write(const char *path, const gb_checkpoint_info *info, const uint64_t *seg_offsets,
                     const double *m_per_system, const double *x_aos, const double *v_aos, std::string &err);

// Fills *info from the header. When any array is given the whole body is
// read, the check word verified and the given arrays filled: seg_offsets
// (nsys + 1 entries) and m_per_system (nsys) for nsys_cap systems at most,
// x_aos and v_aos (3n each) for n_cap particles at most.
int checkpoint_read(const char *path, gb_checkpoint_info *info, uint64_t *seg_offsets, double *m_per_system,
                    size_t nsys_cap, double *x_aos, double *v_aos, size_t n_cap, std::string &err);

}  // namespace gb
