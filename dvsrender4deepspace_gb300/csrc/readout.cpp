// Finite FIFO event readout with the semantics of the reference's
// EventReadout (src/event_readout.cpp:6-34): a batch is ordered by
// (timestamp, y, x); before each arrival the completions due by its time are
// released; with bandwidth B an accepted event completes at
// max(available, t) + 1/B and is delivered at completion + latency; a batch
// arriving while `capacity` events are pending is dropped.  bandwidth <= 0
// passes events straight through.
#include <algorithm>

#include "dvs_internal.h"

namespace dvsgb {

void Readout::submit(std::vector<HostEvent> &batch, double now, std::vector<HostEvent> &ready) {
  std::stable_sort(batch.begin(), batch.end(), [](const HostEvent &a, const HostEvent &b) {
    if (a.t != b.t) return a.t < b.t;
    if (a.y != b.y) return a.y < b.y;
    return a.x < b.x;
  });
  for (const HostEvent &e : batch) {
    while (head_ < queue_.size() && queue_[head_].ready_time <= e.t) ready.push_back(queue_[head_++].event);
    if (bandwidth_ <= 0) {
      ready.push_back(e);
      continue;
    }
    if (queue_.size() - head_ >= capacity_) {
      ++dropped_;
      continue;
    }
    const double completed = std::max(available_, e.t) + 1.0 / bandwidth_;
    available_ = completed;
    HostEvent delivered = e;
    delivered.t = completed + latency_;
    queue_.push_back({completed + latency_, delivered});
    peak_ = std::max(peak_, queue_.size() - head_);
  }
  while (head_ < queue_.size() && queue_[head_].ready_time <= now) ready.push_back(queue_[head_++].event);
  if (head_ > 4096 && head_ * 2 > queue_.size()) {  // compact the consumed prefix
    queue_.erase(queue_.begin(), queue_.begin() + head_);
    head_ = 0;
  }
}

void Readout::drain(std::vector<HostEvent> &ready) {
  while (head_ < queue_.size()) ready.push_back(queue_[head_++].event);
  queue_.clear();
  head_ = 0;
}

}  // namespace dvsgb
