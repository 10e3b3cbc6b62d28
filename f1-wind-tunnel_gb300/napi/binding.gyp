{
  "targets": [{
    "target_name": "wt_napi",
    "sources": ["wt_napi.c"],
    "include_dirs": ["../../include"],
    "libraries": ["-L<(module_root_dir)/../_build", "-lwt", "-Wl,-rpath,<(module_root_dir)/../_build"]
  }]
}
