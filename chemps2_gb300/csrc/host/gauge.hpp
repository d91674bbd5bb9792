// Gauge changes of MPS site tensors on the host (CheMPS2/TensorT.cpp:188-389 and
// CheMPS2/DMRGtechnics.cpp:276-322): left normalisation by QR per right symmetry sector
// (T convention, no spin factors) with R multiplied into the next site from the left, and
// right normalisation by LQ per left symmetry sector in the U convention (blocks scaled by
// sqrt((2S_R + 1) / (2S_L + 1)) before and the inverse after) with L multiplied into the
// previous site from the right. Householder reflections with the LAPACK dgeqr2 / dorg2r
// conventions; the tensors are the column-major blocks of MpsLayout.
#pragma once

#include <vector>

#include "chemps2/SyBookkeeper.h"
#include "layout.hpp"

namespace c2g {

// QR of the m x n column-major matrix a (m >= 1, n >= 1): on return q (m x n) holds the
// first min(m, n) columns of Q (the others zero) and r (n x n) the upper triangle of R
// (rows >= min(m, n) zero).
void householder_qr(int m, int n, const std::vector<double>& a, std::vector<double>& q, std::vector<double>& r);

// Left-normalises `data` (the tensor of `site`); with `next` / `next_lay` non-null, the R
// factors multiply the next site's blocks from the left (DMRG::left_normalize).
void left_normalize(const CheMPS2::SyBookkeeper& bk, int site, const MpsLayout& lay, std::vector<double>& data,
                    const MpsLayout* next_lay = nullptr, std::vector<double>* next = nullptr);

// Right-normalises `data` (the tensor of `site`); with `prev` / `prev_lay` non-null, the L
// factors multiply the previous site's blocks from the right (DMRG::right_normalize).
void right_normalize(const CheMPS2::SyBookkeeper& bk, int site, const MpsLayout& lay, std::vector<double>& data,
                     const MpsLayout* prev_lay = nullptr, std::vector<double>* prev = nullptr);

}  // namespace c2g
