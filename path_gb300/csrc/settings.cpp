// render::Settings defaults, the YAML settings reader and WorkDivision.
//
// Defaults follow include/render/settings.h:27-45 and the settings structs
// it names; the reader accepts the reference's cereal-YAML layout
// (src/render/config_io.cpp:14-35, configs/benchmark.yaml): tagged unions
// are written {type: <Enum>, value: {...}}.
#include "settings.h"

#include "workdiv.h"

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <vector>

namespace pg {

void default_settings(path_settings &s) {
  std::memset(&s, 0, sizeof(s));
  s.kernel_approach = PATH_KERNEL_MEGA;
  s.max_blocks_per_launch_gpu = 4096;
  s.max_blocks_per_launch_cpu = 128;
  s.render_work_division = {256, 32, 0, 8, 16384, 0.5f, 32};
  s.reduce_work_division = {256, 256, 0, 8, 16384, 0.5f, 32};
  s.overlap_threshold = 1e-5f;
  s.use_spatial_splits = 0;
  s.traversal_per_intersect_cost = 0.5f;
  s.target_objects = 4;
  s.light_sampler = PATH_LIGHT_RANDOM_TRIANGLE;
  s.binary_search_threshold = 1073741823u;
  s.dir_sampler = PATH_DIR_BSDF;
  s.term_prob = PATH_TERM_MULTIPLIER_FUNC;
  s.term_prob_prob = 0.5f;
  s.term_prob_iters = 1;
  s.term_prob_exp = 50.0f;
  s.term_prob_min_prob = 0.1f;
  s.rng = PATH_RNG_SOBEL;
  s.max_sample_size = 256;
  s.back_cull_emission = 1;
  s.traversal = PATH_TRAVERSAL_WIDE8;
  s.persistent_ctas_per_sm = 0;
  s.count_work = 0;
}

namespace {

// minimal YAML: block mappings by indentation, "key: scalar", "key: {}" and
// one-line flow mappings {a: 1, b: 2}; comments start with '#'
struct YNode {
  std::string scalar;
  std::map<std::string, std::unique_ptr<YNode>> map;
  bool is_map = false;
};

std::string trim(const std::string &s) {
  size_t a = s.find_first_not_of(" \t\r");
  if (a == std::string::npos) {
    return "";
  }
  size_t b = s.find_last_not_of(" \t\r");
  return s.substr(a, b - a + 1);
}

std::string strip_comment(const std::string &line) {
  bool in_quote = false;
  for (size_t i = 0; i < line.size(); ++i) {
    if (line[i] == '"' || line[i] == '\'') {
      in_quote = !in_quote;
    }
    if (line[i] == '#' && !in_quote && (i == 0 || line[i - 1] == ' ' || line[i - 1] == '\t')) {
      return line.substr(0, i);
    }
  }
  return line;
}

bool parse_flow(const std::string &text, YNode &out, std::string &err) {
  // text is "{...}"
  out.is_map = true;
  std::string body = trim(text.substr(1, text.size() - 2));
  if (body.empty()) {
    return true;
  }
  // split on commas at depth 0
  int depth = 0;
  size_t start = 0;
  std::vector<std::string> parts;
  for (size_t i = 0; i <= body.size(); ++i) {
    if (i == body.size() || (body[i] == ',' && depth == 0)) {
      parts.push_back(trim(body.substr(start, i - start)));
      start = i + 1;
    } else if (body[i] == '{') {
      ++depth;
    } else if (body[i] == '}') {
      --depth;
    }
  }
  for (const std::string &p : parts) {
    size_t c = p.find(':');
    if (c == std::string::npos) {
      err = "flow mapping entry without ':': " + p;
      return false;
    }
    std::string k = trim(p.substr(0, c));
    std::string v = trim(p.substr(c + 1));
    auto child = std::make_unique<YNode>();
    if (!v.empty() && v[0] == '{') {
      if (!parse_flow(v, *child, err)) {
        return false;
      }
    } else {
      child->scalar = v;
    }
    out.map[k] = std::move(child);
  }
  return true;
}

bool parse_yaml(const std::string &text, YNode &root, std::string &err) {
  std::istringstream in(text);
  std::string raw;
  struct Frame {
    int indent;
    YNode *node;
  };
  root.is_map = true;
  std::vector<Frame> stack{{-1, &root}};
  YNode *pending = nullptr; // key with empty value awaiting a nested block
  int pending_indent = -1;
  int line_no = 0;
  while (std::getline(in, raw)) {
    ++line_no;
    std::string line = strip_comment(raw);
    if (trim(line).empty()) {
      continue;
    }
    int indent = 0;
    while (indent < (int)line.size() && line[indent] == ' ') {
      ++indent;
    }
    std::string content = trim(line);
    if (content == "---") {
      continue;
    }
    if (pending) {
      if (indent > pending_indent) {
        pending->is_map = true;
        stack.push_back({indent, pending});
      }
      pending = nullptr;
    }
    while (stack.size() > 1 && indent < stack.back().indent) {
      stack.pop_back();
    }
    if (stack.size() > 1 && indent != stack.back().indent) {
      err = "bad indentation at line " + std::to_string(line_no);
      return false;
    }
    if (stack.size() == 1) {
      stack.back().indent = -1;
    }
    size_t c = content.find(':');
    if (c == std::string::npos) {
      err = "expected 'key: value' at line " + std::to_string(line_no);
      return false;
    }
    std::string key = trim(content.substr(0, c));
    std::string value = trim(content.substr(c + 1));
    auto child = std::make_unique<YNode>();
    YNode *cp = child.get();
    if (value.empty()) {
      pending = cp;
      pending_indent = indent;
    } else if (value[0] == '{') {
      if (value.back() != '}' || !parse_flow(value, *child, err)) {
        if (err.empty()) {
          err = "unterminated flow mapping at line " + std::to_string(line_no);
        }
        return false;
      }
    } else {
      if (value.size() >= 2 && (value[0] == '"' || value[0] == '\'')) {
        value = value.substr(1, value.size() - 2);
      }
      child->scalar = value;
    }
    Frame &top = stack.back();
    if (stack.size() == 1 && top.indent == -1) {
      // first-level keys define the base indentation
    }
    top.node->map[key] = std::move(child);
    if (stack.size() == 1) {
      // keep root indentation loose
    }
  }
  return true;
}

const YNode *get(const YNode *n, const char *key) {
  if (!n || !n->is_map) {
    return nullptr;
  }
  auto it = n->map.find(key);
  return it == n->map.end() ? nullptr : it->second.get();
}

bool read_bool(const YNode *n, uint32_t &out, std::string &err) {
  if (!n) {
    return true;
  }
  if (n->scalar == "true" || n->scalar == "True" || n->scalar == "1") {
    out = 1;
  } else if (n->scalar == "false" || n->scalar == "False" || n->scalar == "0") {
    out = 0;
  } else {
    err = "expected a boolean, got '" + n->scalar + "'";
    return false;
  }
  return true;
}

bool read_u32(const YNode *n, uint32_t &out, std::string &err) {
  if (!n) {
    return true;
  }
  char *end = nullptr;
  unsigned long v = std::strtoul(n->scalar.c_str(), &end, 10);
  if (end == n->scalar.c_str() || *end != '\0') {
    err = "expected an unsigned integer, got '" + n->scalar + "'";
    return false;
  }
  out = (uint32_t)v;
  return true;
}

// a boolean (false / true = 0 / 1) or an unsigned number
bool read_mode(const YNode *n, uint32_t &out, std::string &err) {
  if (n && (n->scalar == "true" || n->scalar == "True" || n->scalar == "false" ||
            n->scalar == "False")) {
    return read_bool(n, out, err);
  }
  return read_u32(n, out, err);
}

bool read_f32(const YNode *n, float &out, std::string &err) {
  if (!n) {
    return true;
  }
  char *end = nullptr;
  float v = std::strtof(n->scalar.c_str(), &end);
  if (end == n->scalar.c_str() || *end != '\0') {
    err = "expected a number, got '" + n->scalar + "'";
    return false;
  }
  out = v;
  return true;
}

bool read_wd(const YNode *n, path_work_division_settings &w, std::string &err) {
  if (!n) {
    return true;
  }
  return read_u32(get(n, "block_size"), w.block_size, err) &&
         read_u32(get(n, "target_x_block_size"), w.target_x_block_size, err) &&
         read_bool(get(n, "force_target_samples"), w.force_target_samples, err) &&
         read_u32(get(n, "forced_target_samples_per_thread"),
                  w.forced_target_samples_per_thread, err) &&
         read_u32(get(n, "base_num_threads"), w.base_num_threads, err) &&
         read_f32(get(n, "samples_per_thread_scaling_power"),
                  w.samples_per_thread_scaling_power, err) &&
         read_u32(get(n, "max_samples_per_thread"), w.max_samples_per_thread, err);
}

bool read_type(const YNode *n, const char *const *names, uint32_t count,
               uint32_t &out, std::string &err) {
  const YNode *t = get(n, "type");
  if (!t) {
    return true;
  }
  for (uint32_t i = 0; i < count; ++i) {
    if (t->scalar == names[i]) {
      out = i;
      return true;
    }
  }
  err = "unknown type '" + t->scalar + "'";
  return false;
}

} // namespace

bool settings_from_yaml_text(const std::string &text, path_settings &s,
                             std::string &err) {
  default_settings(s);
  YNode root;
  if (!parse_yaml(text, root, err)) {
    return false;
  }
  const YNode *st = get(&root, "settings");
  if (!st) {
    st = &root;
  }
  // kernel approach
  if (const YNode *ka = get(st, "kernel_approach")) {
    static const char *kNames[] = {"MegaKernel", "Streaming"};
    if (!read_type(ka, kNames, 2, s.kernel_approach, err)) {
      return false;
    }
    const YNode *v = get(ka, "value");
    const YNode *cs = get(v, "computation_settings");
    if (!read_u32(get(cs, "max_blocks_per_launch_gpu"), s.max_blocks_per_launch_gpu, err) ||
        !read_u32(get(cs, "max_blocks_per_launch_cpu"), s.max_blocks_per_launch_cpu, err) ||
        !read_wd(get(cs, "render_work_division"), s.render_work_division, err) ||
        !read_wd(get(cs, "reduce_work_division"), s.reduce_work_division, err)) {
      return false;
    }
    const YNode *iis = get(v, "individually_intersectable_settings");
    const YNode *accel = get(iis, "accel");
    if (!accel) {
      accel = get(v, "accel");
    }
    if (accel) {
      static const char *aNames[] = {"SBVH"};
      uint32_t dummy = 0;
      if (!read_type(accel, aNames, 1, dummy, err)) {
        return false;
      }
      const YNode *av = get(accel, "value");
      const YNode *bs = get(av, "bvh_settings");
      if (!read_f32(get(av, "overlap_threshold"), s.overlap_threshold, err) ||
          !read_bool(get(av, "use_spatial_splits"), s.use_spatial_splits, err) ||
          !read_f32(get(bs, "traversal_per_intersect_cost"),
                    s.traversal_per_intersect_cost, err) ||
          !read_u32(get(bs, "target_objects"), s.target_objects, err)) {
        return false;
      }
    }
  }
  if (const YNode *ls = get(st, "light_sampler")) {
    static const char *names[] = {"RandomTriangle", "NoLightSampling"};
    if (!read_type(ls, names, 2, s.light_sampler, err) ||
        !read_u32(get(get(ls, "value"), "binary_search_threshold"),
                  s.binary_search_threshold, err)) {
      return false;
    }
  }
  if (const YNode *ds = get(st, "dir_sampler")) {
    static const char *names[] = {"BSDF", "Uniform"};
    if (!read_type(ds, names, 2, s.dir_sampler, err)) {
      return false;
    }
  }
  if (const YNode *tp = get(st, "term_prob")) {
    static const char *names[] = {"Constant", "NIters", "MultiplierFunc", "Normalize"};
    if (!read_type(tp, names, 4, s.term_prob, err)) {
      return false;
    }
    const YNode *v = get(tp, "value");
    if (!read_f32(get(v, "prob"), s.term_prob_prob, err) ||
        !read_u32(get(v, "iters"), s.term_prob_iters, err) ||
        !read_f32(get(v, "exp"), s.term_prob_exp, err) ||
        !read_f32(get(v, "min_prob"), s.term_prob_min_prob, err)) {
      return false;
    }
  }
  if (const YNode *rng = get(st, "rng")) {
    static const char *names[] = {"Sobel", "Uniform"};
    if (!read_type(rng, names, 2, s.rng, err) ||
        !read_u32(get(get(rng, "value"), "max_sample_size"), s.max_sample_size, err)) {
      return false;
    }
  }
  if (const YNode *re = get(st, "rendering_equation_settings")) {
    if (!read_bool(get(re, "back_cull_emission"), s.back_cull_emission, err)) {
      return false;
    }
  }
  // GB300 knobs (no reference counterpart)
  if (const YNode *g = get(st, "gb300")) {
    if (const YNode *t = get(g, "traversal")) {
      if (t->scalar == "Binary") {
        s.traversal = PATH_TRAVERSAL_BINARY;
      } else if (t->scalar == "Wide8") {
        s.traversal = PATH_TRAVERSAL_WIDE8;
      } else {
        err = "unknown traversal '" + t->scalar + "'";
        return false;
      }
    }
    if (!read_u32(get(g, "persistent_ctas_per_sm"), s.persistent_ctas_per_sm, err) ||
        !read_u32(get(g, "trace_min_blocks"), s.trace_min_blocks, err) ||
        !read_bool(get(g, "count_work"), s.count_work, err) ||
        !read_bool(get(g, "time_kernels"), s.time_kernels, err) ||
        !read_mode(get(g, "gpu_build"), s.gpu_build, err) ||
        !read_u32(get(g, "wavefront_slots_log2"), s.wavefront_slots_log2, err) ||
        !read_u32(get(g, "trace_staged_nodes"), s.trace_staged_nodes, err)) {
      return false;
    }
  }
  return true;
}

bool settings_from_yaml_file(const std::string &path, path_settings &s,
                             std::string &err) {
  std::ifstream f(path);
  if (!f) {
    err = "cannot open settings file " + path;
    return false;
  }
  std::stringstream ss;
  ss << f.rdbuf();
  return settings_from_yaml_text(ss.str(), s, err);
}

static bool is_pow2(uint32_t n) { return n != 0 && (n & (n - 1)) == 0; }

static uint32_t closest_pow2(uint32_t n) {
  if (n == 0) {
    return 1;
  }
  uint32_t place = 31 - (uint32_t)__builtin_clz(n);
  uint32_t lower = 1u << place;
  if (place == 31) {
    return lower;
  }
  uint32_t upper = lower << 1;
  return (n - lower <= upper - n) ? lower : upper;
}

// WorkDivision constructor (src/kernel/work_division.cpp:12-69)
bool make_workdiv(const path_work_division_settings &s, uint32_t samples_per,
                  uint32_t x_dim, uint32_t y_dim, WorkDiv &o) {
  if (s.block_size % 32 != 0 || !is_pow2(s.block_size) ||
      !is_pow2(s.target_x_block_size) || samples_per == 0) {
    return false;
  }
  o.block_size = s.block_size;
  double target;
  if (s.force_target_samples) {
    target = s.forced_target_samples_per_thread;
  } else {
    double total = ((double)samples_per * x_dim) * y_dim;
    double ratio = total / s.base_num_threads;
    double base = std::pow(ratio, (double)s.samples_per_thread_scaling_power);
    target = std::min(base, (double)s.max_samples_per_thread);
  }
  uint32_t n_threads = closest_pow2((uint32_t)std::round((double)samples_per / target));
  o.base_samples_per_thread = samples_per / n_threads;
  o.n_threads_per_unit_extra = samples_per - o.base_samples_per_thread * n_threads;
  o.sample_block_size = std::min(n_threads, o.block_size);
  uint32_t xy = o.block_size / o.sample_block_size;
  o.x_block_size = std::min(xy, s.target_x_block_size);
  o.y_block_size = xy / o.x_block_size;
  o.num_sample_blocks = n_threads / o.sample_block_size;
  o.num_x_blocks = (x_dim + o.x_block_size - 1) / o.x_block_size;
  o.num_y_blocks = (y_dim + o.y_block_size - 1) / o.y_block_size;
  o.x_dim = x_dim;
  o.y_dim = y_dim;
  return (uint64_t)o.num_sample_blocks * x_dim * y_dim < 0xffffffffull;
}

} // namespace pg
