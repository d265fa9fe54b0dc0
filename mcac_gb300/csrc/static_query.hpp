// Batched contact queries with no device allocation (static_query.cu).
#pragma once
#include <cstdint>
#include <string>

#include "../../include/mcacg.h"
#include "device_box.hpp"

namespace mcacg {

// The queries of HostBox::distance_to_next_contacts on 'dev' (n_alive live
// aggregates), with every device buffer in a file-scope __device__ array.
int query_batch_static(DeviceBox &dev, int n_alive, int n, const int64_t *sources, const double *dirs,
                       const double *dists, mcacg_contact *out, std::string *err);

}  // namespace mcacg
