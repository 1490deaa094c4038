{
  "targets": [
    {
      "target_name": "gs3d_node",
      "sources": ["gs3d_node.c"],
      "include_dirs": ["../../include", "<!(echo ${CUDA_HOME:-/usr/local/cuda})/include"],
      "libraries": [
        "-L<(module_root_dir)/../_build", "-lgs3d",
        "-L<!(echo ${CUDA_HOME:-/usr/local/cuda})/lib64", "-lcudart",
        "-Wl,-rpath,<(module_root_dir)/../_build"
      ],
      "cflags": ["-std=c11", "-Wall", "-Wextra"]
    }
  ]
}
