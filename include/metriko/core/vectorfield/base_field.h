//
// Restates parts of metriko (https://github.com/komietty/metriko),
// Copyright (C) 2025 Saki Komikado <komietty@gmail.com>.
// This Source Code Form is subject to the terms of the Mozilla Public License v.2.0
// (https://mozilla.org/MPL/2.0/).
//
// metriko-gb300: vector-field container (reference: include/metriko/core/vectorfield/base_field.h:10-23).
//
#ifndef METRIKO_BASE_FIELD_H
#define METRIKO_BASE_FIELD_H
#include "metriko/core/hmesh/hmesh.h"

namespace metriko {
    class BaseVectorField {
    public:
        const Hmesh& mesh;
        const int rosyN;
        MatXc field;        // nF x N
        VecXc connection;   // nE
        VecXc compressed;   // nF (the eigenvector of the smoothest field)
        VecXi matching;     // nE
        VecXi singular;     // nV
        BaseVectorField(const Hmesh& m, const int n) : mesh(m), rosyN(n) {}
    };

    enum class FieldType { UnSpecified, Smoothest, CurvatureAligned };
    enum class MatchingType { Principal, Curl };
}

#endif
