{
  "targets": [{
    "target_name": "webgs",
    "sources": ["addon.cc"],
    "include_dirs": ["../../include"],
    "libraries": ["-L<(module_root_dir)/../lib", "-lwebgs", "-Wl,-rpath,<(module_root_dir)/../lib"],
    "cflags_cc": ["-std=c++17"]
  }]
}
