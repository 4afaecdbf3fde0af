// Stand-in for the subset of spdlog the reference's MACIS headers call:
// named loggers in a process-wide registry (get, stdout_color_mt,
// null_logger_mt, drop_all) whose level methods work and whose message
// methods discard their arguments (the fixture builds need no log output).
#pragma once
// the real library's headers bring these in; the reference relies on that
#include <atomic>
#include <chrono>
#include <cstdio>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <string>

namespace spdlog {
namespace level {
enum level_enum { trace = 0, debug, info, warn, err, critical, off };
}

class logger {
 public:
  explicit logger(std::string name) : name_(std::move(name)) {}
  template <class... A> void trace(A&&...) {}
  template <class... A> void debug(A&&...) {}
  template <class... A> void info(A&&...) {}
  template <class... A> void warn(A&&...) {}
  template <class... A> void error(A&&...) {}
  template <class... A> void critical(A&&...) {}
  bool should_log(level::level_enum l) const { return l >= level_; }
  level::level_enum level() const { return level_; }
  void set_level(level::level_enum l) { level_ = l; }
  void flush_on(level::level_enum) {}
  void flush() {}
  const std::string& name() const { return name_; }

 private:
  std::string name_;
  level::level_enum level_ = level::info;
};

namespace detail {
inline std::mutex& registry_mutex() {
  static std::mutex m;
  return m;
}
inline std::map<std::string, std::shared_ptr<logger>>& registry() {
  static std::map<std::string, std::shared_ptr<logger>> r;
  return r;
}
inline std::shared_ptr<logger> make(const std::string& name) {
  std::lock_guard<std::mutex> lk(registry_mutex());
  auto& r = registry();
  auto it = r.find(name);
  if (it != r.end()) return it->second;
  auto l = std::make_shared<logger>(name);
  r[name] = l;
  return l;
}
}  // namespace detail

inline std::shared_ptr<logger> get(const std::string& name) {
  std::lock_guard<std::mutex> lk(detail::registry_mutex());
  auto& r = detail::registry();
  auto it = r.find(name);
  return it == r.end() ? nullptr : it->second;
}
inline std::shared_ptr<logger> stdout_color_mt(const std::string& name) { return detail::make(name); }
inline std::shared_ptr<logger> null_logger_mt(const std::string& name) { return detail::make(name); }
template <class... A> void trace(A&&...) {}
template <class... A> void debug(A&&...) {}
template <class... A> void info(A&&...) {}
template <class... A> void warn(A&&...) {}
template <class... A> void error(A&&...) {}
inline void set_level(level::level_enum) {}
inline void drop(const std::string& name) {
  std::lock_guard<std::mutex> lk(detail::registry_mutex());
  detail::registry().erase(name);
}
inline void drop_all() {
  std::lock_guard<std::mutex> lk(detail::registry_mutex());
  detail::registry().clear();
}
}  // namespace spdlog
