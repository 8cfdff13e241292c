"""GB300-native particle<->grid interpolation with the Cabana::Grid p2g/g2p
operator API.

Submodules:
  mesh   -- host-side mesh geometry (no GPU needed)
  grid   -- Cabana::Grid-style Array / Halo / functors / p2g / g2p over torch
            CUDA tensors, calling libcgx.so through its C ABI
  core   -- LinkedCellList / BinningData / permute / binByKey / sortByKey
"""
