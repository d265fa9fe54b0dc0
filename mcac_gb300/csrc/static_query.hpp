// Batched contact queries with no device allocation (static_query.cu).
#pragma once
#include <cstdint>
#include <string>

#include "../../include/mcacg.h"
#include "device_box.hpp"

namespace mcacg {

// The queries of HostBox::distance_to_next_contacts on 'dev', from the
// moving aggregates' slots, with every device buffer in a file-scope
// __device__ array. out[k] gets the distance and spheres of query k, and the
// hit aggregate's slot in other_aggregate (-1 if none); moving_aggregate is
// left at -1: the caller turns slots into labels.
int query_batch_static(DeviceBox &dev, int n, const int *slots, const double *dirs, const double *dists,
                       mcacg_contact *out, std::string *err);

}  // namespace mcacg
