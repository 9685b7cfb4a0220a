// json_args.cpp -- reader for the --args_path JSON file: one flat object whose
// values are numbers, strings, booleans or null (the reference reads it with
// nlohmann::json and args.value(key, default), e.g. src/one_to_one.hpp:185).
#include <cctype>
#include <fstream>
#include <sstream>

#include "cross.hpp"

namespace cross {

namespace {

struct parser {
  const std::string& s;
  size_t i = 0;

  explicit parser(const std::string& text) : s(text) {}

  void ws() {
    while (i < s.size() && std::isspace((unsigned char)s[i])) ++i;
  }
  [[noreturn]] void error(const std::string& what) {
    throw argument_error("invalid JSON in algorithm arguments: " + what + " at offset " + std::to_string(i));
  }
  char peek() {
    ws();
    return i < s.size() ? s[i] : '\0';
  }
  void expect(char c) {
    if (peek() != c) error(std::string("expected '") + c + "'");
    ++i;
  }
  std::string string_lit() {
    expect('"');
    std::string out;
    while (i < s.size() && s[i] != '"') {
      if (s[i] == '\\' && i + 1 < s.size()) {
        ++i;
        switch (s[i]) {
          case 'n': out.push_back('\n'); break;
          case 't': out.push_back('\t'); break;
          default: out.push_back(s[i]); break;
        }
      } else {
        out.push_back(s[i]);
      }
      ++i;
    }
    if (i >= s.size()) error("unterminated string");
    ++i;
    return out;
  }
  std::string scalar() {
    char c = peek();
    if (c == '"') return string_lit();
    size_t st = i;
    while (i < s.size() && (std::isalnum((unsigned char)s[i]) || s[i] == '-' || s[i] == '+' || s[i] == '.')) ++i;
    if (st == i) error("expected a value");
    return s.substr(st, i - st);
  }
};

}  // namespace

json_args json_args::parse_file(const std::string& path) {
  std::ifstream in(path);
  if (!in) throw argument_error("cannot open algorithm arguments file " + path);
  std::stringstream ss;
  ss << in.rdbuf();
  const std::string text = ss.str();
  parser p(text);
  json_args out;
  p.expect('{');
  if (p.peek() == '}') return out;
  for (;;) {
    std::string key = p.string_lit();
    p.expect(':');
    if (p.peek() == '{' || p.peek() == '[') p.error("nested values are not supported");
    out.values[key] = p.scalar();
    char c = p.peek();
    if (c == ',') {
      ++p.i;
      continue;
    }
    if (c == '}') break;
    p.error("expected ',' or '}'");
  }
  return out;
}

long long json_args::get_int(const std::string& key, long long def) const {
  auto it = values.find(key);
  if (it == values.end() || it->second == "null") return def;
  try {
    size_t pos = 0;
    long long v = std::stoll(it->second, &pos);
    if (pos != it->second.size()) throw std::invalid_argument(key);
    return v;
  } catch (const std::exception&) {
    throw argument_error("argument " + key + " must be an integer, got " + it->second);
  }
}

std::string json_args::get_str(const std::string& key, const std::string& def) const {
  auto it = values.find(key);
  return it == values.end() || it->second == "null" ? def : it->second;
}

bool json_args::get_bool(const std::string& key, bool def) const {
  auto it = values.find(key);
  if (it == values.end() || it->second == "null") return def;
  if (it->second == "true") return true;
  if (it->second == "false") return false;
  throw argument_error("argument " + key + " must be a boolean, got " + it->second);
}

}  // namespace cross
