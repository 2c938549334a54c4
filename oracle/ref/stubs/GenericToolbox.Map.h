// Stand-in for the two GenericToolbox helpers BarlowBeestonBanff2022.h names.
#ifndef GW_REF_STUB_GT_MAP_H
#define GW_REF_STUB_GT_MAP_H
#include <map>
#include <mutex>

namespace GenericToolbox {
template <typename K, typename M>
bool isIn(const K& key, const M& map) {
  return map.find(key) != map.end();
}
// a member that copies as a fresh default object
template <typename T>
struct NoCopyWrapper : T {
  NoCopyWrapper() = default;
  NoCopyWrapper(const NoCopyWrapper&) : T() {}
  NoCopyWrapper& operator=(const NoCopyWrapper&) { return *this; }
};
}  // namespace GenericToolbox
#endif
