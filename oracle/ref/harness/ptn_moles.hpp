// Per-cell PTN moles for the harness's decks (test infrastructure, shared by
// the dump harness and the binding driver).
#pragma once
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <string>
#include <vector>

// The reference's grid distributor refuses more than 30 per-cell input arrays
// (src/Reservoir.cpp:38-66), so a PTN start with more than four hydrocarbon
// components cannot carry its COMPM-* arrays through the deck.  Decks written
// for this harness therefore leave COMPM-* out and place the per-cell moles
// (cell-major, hydrocarbons then water) in "<deck>.ptn_ni"; they are copied
// into the bulk initializer exactly where the deck reader would have put them.
inline void inject_ptn_moles(Reservoir& rs, const std::string& deck)
{
    const std::string path = deck + ".ptn_ni";
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) return;
    const OCP_USI nb = rs.bulk.vs.nb;
    const USI     nc = rs.bulk.vs.nc;
    std::vector<double> buf(static_cast<size_t>(nb) * nc);
    if (std::fread(buf.data(), sizeof(double), buf.size(), f) != buf.size()) {
        std::cerr << "short ptn_ni file\n";
        std::exit(6);
    }
    std::fclose(f);
    auto& Ni = rs.bulk.INITm.GetNi();
    Ni.assign(nc, std::vector<OCP_DBL>(nb));
    for (OCP_USI n = 0; n < nb; n++)
        for (USI i = 0; i < nc; i++) Ni[i][n] = buf[static_cast<size_t>(n) * nc + i];
}

