//
// Restates parts of metriko (https://github.com/komietty/metriko),
// Copyright (C) 2025 Saki Komikado <komietty@gmail.com>.
// This Source Code Form is subject to the terms of the Mozilla Public License v.2.0
// (https://mozilla.org/MPL/2.0/).
//
// metriko-gb300: iterative rounding entry point.
//
// Replaces metriko include/metriko/core/igm/iterative_rounding/iter_rounding.h:33-113 (and the
// NaiveIntegration / SeamlessIntegration / LMSolver / CholeskyWrapper machinery under it).  The
// reference's argument list (fixedIdcs, fixedVals, singularIdcs, integerIdcs, length, Cfull,
// G2, ...) is carried by mtk_igm_desc in the factored form the device operator uses
// (cut-mesh faces and positions, the W map, UFull's kernel block); the whole loop runs on the
// GPU through mtk_iterative_rounding.  Returns false when the post-rounding integrality check
// fails, as the reference does.
//
#ifndef METRIKO_ITER_ROUNDING_H
#define METRIKO_ITER_ROUNDING_H
#include "metriko/core/common/typedef.h"
#include "metriko/gpu/device.h"

namespace metriko {
    inline bool iterative_rounding(const mtk_igm_desc& d, VecXd& fullx, VecXd& naivex, std::vector<int>& fixOrder,
                                   std::vector<int>& fixVals) {
        fullx = VecXd(d.nFull);
        naivex = VecXd(d.nFull);
        const int cap = std::max(1, d.nSingular + d.nInteger);
        fixOrder.assign(cap, -1);
        fixVals.assign(cap, 0);
        int nfix = 0;
        int s = mtk_iterative_rounding(gpu::context(), &d, &gpu::options().solve, fullx.data(), fixOrder.data(),
                                       fixVals.data(), &nfix, naivex.data(), &gpu::stats());
        fixOrder.resize(std::min(nfix, cap));
        fixVals.resize(std::min(nfix, cap));
        if (s == MTK_ERR_ROUNDING) return false;
        gpu::check(s, "mtk_iterative_rounding");
        return true;
    }
}

#endif
