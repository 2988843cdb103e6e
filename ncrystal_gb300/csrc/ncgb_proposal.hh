// Tables of the learned beta proposal (ncgb_proposal.cc).
#ifndef NCGB_PROPOSAL_HH
#define NCGB_PROPOSAL_HH

#include "ncgb_host.hh"

#include <vector>

namespace ncgb {

  struct Proposal {
    std::vector<ncgb_lp_hdr> hdr;    // [ne]
    std::vector<ncgb_lp_slot> slot;  // [ne * NCGB_LP_K]
    std::vector<ncgb_lp_cell> cell;  // [ne * NCGB_LP_K]
    std::vector<ncgb_lp_seg> seg;    // linear pieces of all intervals
  };

  // 's' with host pointers; knots[ne * nknots]: asinh(beta) knots per egrid
  // point; allowed[ne] (may be null): egrid points inside the network's trained
  // range.  Egrid points with an acceptance ratio below min_accept stay
  // disabled (plain inversion).
  Proposal buildProposal( const ncgb_sab_view& s, const float* knots, int nknots, const unsigned char* allowed,
                          double min_accept );
}

#endif
