// main.cpp -- `cross`: command-line front end with the reference CLI's
// commands and options (src/main.cpp:465-683, README "CLI commands").
//
//   cross [global options] list
//   cross [global options] run [run options] <alg> <ref_path> <target_path>
//   cross [global options] validate [validate options] <template_data_path> <validate_data_path>...
//   cross [global options] input <alg_type> <rows> <columns> <left_matrices> <right_matrices>
//
// Exit codes: 0 success, 1 command-line or algorithm-argument errors,
// 2 other exceptions, 3 failure of a computation step.
#include <cstdlib>
#include <iostream>
#include <string>
#include <vector>

#include "cross.hpp"

using namespace cross;

namespace {

struct usage_error : std::runtime_error {
  using std::runtime_error::runtime_error;
};

void print_help(std::ostream& out, const std::string& name) {
  out << "Usage: " << name << " [global options] command [command options]\n";
  out << "Commands: \n";
  out << "\t" << name << " [global options] list\n";
  out << "\t" << name << " [global options] run [run options] <alg> <ref_path> <target_path>\n";
  out << "\t" << name << " [global options] validate [validate options] <validate_data_path> <template_data_path>\n";
  out << "\t" << name
      << " [global options] input [input options] <alg_type> <rows> <columns> <left_matrices> <right_matrices>\n";
  out << "Global options:\n"
         "  -h [ --help ]               display this help and exit\n"
         "Validate options:\n"
         "  -n [ --normalize ]          Normalize the data to be validated as they are denormalized fft output\n"
         "  -c [ --csv ]                CSV output\n"
         "  -p [ --print_header ]       Print header\n"
         "Run options:\n"
         "  -d [ --data_type ] arg (=single)          Data type to use for computation\n"
         "  -o [ --out ] arg                          Path of the output file to be created\n"
         "  -t [ --times ] arg (=measurements.csv)    File to store the measured times in\n"
         "  -v [ --validate ] [=arg(=)]               If validation of the results should be done and optionally\n"
         "                                            path to a file containing the valid results\n"
         "  -n [ --normalize ]                        If algorithm is fft, normalize the results\n"
         "  -a [ --append ]                           Append time measurements without the header\n"
         "  -p [ --no_progress ]                      Do not print human readable progress\n"
         "  -b [ --benchmark_type ] arg (=None)       Which part should be measured: Compute, CommonSteps,\n"
         "                                            Algorithm\n"
         "  -l [ --outer_loops ] arg (=1)             How many measurements of the computation loop\n"
         "  -m [ --min_time ] arg (=1)                The minimum measurement time, in seconds\n"
         "  --args_path arg                           Path to the JSON file containing arguments for the algorithm\n";
}

// Splits "--name=value" / "-xvalue" forms.
struct token {
  std::string name;  // option name without dashes ("" for positional)
  std::string value;
  bool has_value = false;
  bool is_long = false;
};

token classify(const std::string& a) {
  token t;
  if (a.size() >= 2 && a[0] == '-' && a[1] == '-') {
    t.is_long = true;
    size_t eq = a.find('=');
    t.name = a.substr(2, eq == std::string::npos ? std::string::npos : eq - 2);
    if (eq != std::string::npos) {
      t.value = a.substr(eq + 1);
      t.has_value = true;
    }
  } else if (a.size() >= 2 && a[0] == '-' && !(a[1] >= '0' && a[1] <= '9')) {
    t.name = a.substr(1, 1);
    if (a.size() > 2) {
      t.value = a.substr(2);
      t.has_value = true;
    }
  } else {
    t.value = a;
  }
  return t;
}

std::string long_name(const token& t, const std::vector<std::pair<char, std::string>>& map) {
  if (t.is_long) return t.name;
  for (const auto& m : map)
    if (t.name.size() == 1 && t.name[0] == m.first) return m.second;
  throw usage_error("unrecognised option '-" + t.name + "'");
}

benchmark_type parse_bench(const std::string& s) {
  if (s == "None") return benchmark_type::None;
  if (s == "Compute") return benchmark_type::Compute;
  if (s == "CommonSteps") return benchmark_type::CommonSteps;
  if (s == "Algorithm") return benchmark_type::Algorithm;
  throw usage_error("the argument ('" + s + "') for option '--benchmark_type' is invalid");
}

int cmd_run(const std::vector<std::string>& argv, const std::string& prog) {
  run_args ra;
  std::vector<std::string> pos;
  bool validate_took_value = false;
  const std::vector<std::pair<char, std::string>> shorts = {
      {'d', "data_type"}, {'o', "out"},     {'t', "times"},          {'v', "validate"},    {'n', "normalize"},
      {'a', "append"},    {'p', "no_progress"}, {'b', "benchmark_type"}, {'l', "outer_loops"}, {'m', "min_time"}};
  for (size_t i = 0; i < argv.size(); ++i) {
    token t = classify(argv[i]);
    if (t.name.empty()) {
      pos.push_back(t.value);
      continue;
    }
    const std::string name = long_name(t, shorts);
    auto need_value = [&]() -> std::string {
      if (t.has_value) return t.value;
      if (i + 1 >= argv.size()) throw usage_error("the required argument for option '--" + name + "' is missing");
      return argv[++i];
    };
    if (name == "data_type") ra.data_type = need_value();
    else if (name == "out") {
      std::string v = need_value();
      if (!v.empty()) ra.out_path = v;
    } else if (name == "times") ra.measurements_path = need_value();
    else if (name == "validate") {
      ra.validate = true;
      if (t.has_value) {
        ra.validate_path = t.value;
      } else if (i + 1 < argv.size() && !argv[i + 1].empty() && argv[i + 1][0] != '-') {
        // An optional value: taken when a path follows (see the check below).
        ra.validate_path = argv[++i];
        validate_took_value = true;
      }
    } else if (name == "normalize") ra.normalize = true;
    else if (name == "append") ra.append = true;
    else if (name == "no_progress") ra.progress = false;
    else if (name == "benchmark_type") ra.bench = parse_bench(need_value());
    else if (name == "outer_loops") ra.outer_loops = (size_t)std::stoull(need_value());
    else if (name == "min_time") ra.min_time = std::chrono::nanoseconds((long long)(std::stod(need_value()) * 1e9));
    else if (name == "args_path") ra.args_path = need_value();
    else throw usage_error("unrecognised option '" + argv[i] + "'");
  }
  // "-v <alg> <ref> <target>": the token after -v was the algorithm name.
  if (validate_took_value && pos.size() == 2) {
    pos.insert(pos.begin(), ra.validate_path);
    ra.validate_path.clear();
  }
  if (pos.size() != 3) throw usage_error("run expects <alg> <ref_path> <target_path>");
  ra.alg_name = pos[0];
  ra.ref_path = pos[1];
  ra.target_path = pos[2];
  if (!algorithm_exists(ra.alg_name)) {
    std::cerr << "Unknown algorithm \"" << ra.alg_name << "\", expected one of [";
    const char* sep = "";
    for (const auto& n : algorithm_names()) {
      std::cerr << sep << n;
      sep = ", ";
    }
    std::cerr << "]" << std::endl;
    print_help(std::cerr, prog);
    return 1;
  }
  int ret = run_algorithm(ra);
  if (ret == 1) print_help(std::cerr, prog);
  return ret;
}

int cmd_validate(const std::vector<std::string>& argv) {
  bool normalize = false, csv = false, header = false;
  std::vector<std::string> pos;
  const std::vector<std::pair<char, std::string>> shorts = {{'n', "normalize"}, {'c', "csv"}, {'p', "print_header"}};
  for (const auto& a : argv) {
    token t = classify(a);
    if (t.name.empty()) {
      pos.push_back(t.value);
      continue;
    }
    const std::string name = long_name(t, shorts);
    if (name == "normalize") normalize = true;
    else if (name == "csv") csv = true;
    else if (name == "print_header") header = true;
    else throw usage_error("unrecognised option '" + a + "'");
  }
  if (pos.size() < 2) throw usage_error("validate expects <template_data_path> <validate_data_path>...");
  // validate<double> (src/main.cpp:56-79)
  auto valid = load_csv<double>(pos[0]);
  for (size_t i = 1; i < pos.size(); ++i) {
    if (!csv) std::cout << "Validating " << pos[i] << std::endl;
    auto target = load_csv<double>(pos[i]);
    if (normalize) target = normalize_fft_host(target);
    print_validation(validate_result(target, valid), !csv, i == 1 && header);
  }
  return 0;
}

int cmd_input(const std::vector<std::string>& argv, const std::string& prog) {
  if (argv.size() != 5) throw usage_error("input expects <alg_type> <rows> <columns> <left_matrices> <right_matrices>");
  auto u = [](const std::string& s) {
    long long v = std::stoll(s);
    if (v < 0) throw usage_error("the argument ('" + s + "') is invalid");
    return (uint32_t)v;
  };
  bool known = false;
  bool ok = validate_input_size(argv[0], u(argv[1]), u(argv[2]), u(argv[3]), u(argv[4]), &known);
  if (!known) {
    std::cerr << "Unknown algorithm type \"" << argv[0] << "\", expected one of [n_to_m, n_to_mn, one_to_many, one_to_one]"
              << std::endl;
    print_help(std::cerr, prog);
    return 1;
  }
  std::cout << (ok ? "Valid\n" : "Invalid\n");
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  const std::string prog = argv[0];
  try {
    std::vector<std::string> args(argv + 1, argv + argc);
    size_t ci = 0;
    while (ci < args.size() && !args[ci].empty() && args[ci][0] == '-') {
      if (args[ci] == "-h" || args[ci] == "--help") {
        print_help(std::cout, prog);
        return 0;
      }
      throw usage_error("unrecognised option '" + args[ci] + "'");
    }
    if (ci >= args.size()) {
      print_help(std::cout, prog);
      return 0;
    }
    const std::string cmd = args[ci];
    std::vector<std::string> sub(args.begin() + ci + 1, args.end());
    for (const auto& a : sub)
      if (a == "-h" || a == "--help") {
        print_help(std::cout, prog);
        return 0;
      }
    if (cmd == "run") return cmd_run(sub, prog);
    if (cmd == "validate") return cmd_validate(sub);
    if (cmd == "list") {
      for (const auto& n : algorithm_names()) std::cout << n << "\n";
      return 0;
    }
    if (cmd == "input") return cmd_input(sub, prog);
    if (cmd == "help") {
      print_help(std::cout, prog);
      return 0;
    }
    std::cerr << "Unknown command " << cmd << "\n";
    print_help(std::cerr, prog);
    return 1;
  } catch (usage_error& e) {
    std::cerr << "Invalid commandline options: " << e.what() << std::endl;
    return 1;
  } catch (argument_error& e) {
    std::cerr << "Invalid algorithm argument value: " << e.what() << std::endl;
    return 1;
  } catch (std::invalid_argument& e) {
    std::cerr << "Invalid commandline options: " << e.what() << std::endl;
    return 1;
  } catch (std::exception& e) {
    std::cerr << "Exception occured: " << e.what() << std::endl;
    return 2;
  }
}
