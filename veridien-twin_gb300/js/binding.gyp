{
  "targets": [
    {
      "target_name": "vtwin",
      "sources": ["vtwin_addon.cc"],
      "include_dirs": ["../../include"],
      "libraries": ["-L<(module_root_dir)/../vtwin", "-lvtwin", "-Wl,-rpath,<(module_root_dir)/../vtwin"],
      "cflags_cc": ["-std=c++17", "-O2"]
    }
  ]
}
