// The reference's own pipeline shape, driven by hand over the drop-in
// headers: CudaBlockScheduler -> PcfBlockOp::exec_block per block ->
// download -> BlockResultWriter::scatter.  Prints "ok" when the assembled
// DistanceMatrix / SymmetricMatrix / dense cdist equal the factories' results
// bit for bit.
#include <sbgpu/block_op.hpp>

#include <cstdio>
#include <cstdlib>

#define CHECK(c)                                                                          \
  do {                                                                                    \
    if (!(c)) { std::printf("FAIL %s:%d %s\n", __FILE__, __LINE__, #c); std::exit(1); } \
  } while (0)

static std::vector<sb::Pcf<float, float>> make_pcfs(size_t n, unsigned seed)
{
  std::vector<sb::Pcf<float, float>> out;
  unsigned s = seed;
  auto next = [&s]() { s = s * 1664525u + 1013904223u; return (s >> 8) * (1.0f / 16777216.0f); };
  for (size_t i = 0; i < n; ++i)
  {
    std::vector<sb::TimePoint<float, float>> pts;
    const int len = 1 + (int)(next() * 40);
    float t = 0.f;
    for (int k = 0; k < len; ++k)
    {
      pts.emplace_back(t, k + 1 == len ? 0.f : next() * 4.f - 2.f);
      t += 0.05f + next();
    }
    out.emplace_back(std::move(pts));
  }
  return out;
}

template <typename MatT, typename Op, typename WriterT>
static void run_blocks(MatT& mat, sb::CudaPcfDataManager<float, float>& rows, sb::CudaPcfDataManager<float, float>& cols,
                       Op op, sb::TriangleSkipMode skip, bool lower)
{
  sb::CudaBlockScheduler::Config cfg{};
  cfg.nRows = rows.size();
  cfg.nCols = cols.size();
  cfg.maxOutputElements = 96 * 96;
  cfg.nSplitsHint = 8;
  cfg.triangleMode = lower ? sb::BlockTriangleMode::LowerTriangle : sb::BlockTriangleMode::Full;
  cfg.minBlockSide = 0;
  sb::CudaBlockScheduler sched(cfg);
  sb::PcfBlockOp<float, float, Op> bop(rows, cols, op, 0.f, std::numeric_limits<float>::max(), skip);
  auto storage = bop.init_gpu_storage(0, sched);
  sb::CudaDeviceArray<float> tile(sched.max_row_height() * sched.max_col_width());
  std::vector<float> host(tile.size());
  WriterT writer(mat);
  for (const auto& b : sched.blocks())
  {
    tile.clear();
    bop.exec_block(storage, b, tile, 0);
    tile.download(host.data(), b.rowHeight * b.colWidth);
    writer.scatter(host.data(), b);
  }
}

int main()
{
  const size_t n = 700, m = 230;
  auto pcfs = make_pcfs(n, 7);
  auto others = make_pcfs(m, 11);
  sb::CudaPcfDataManager<float, float> dmgr(pcfs), omgr(others);

  // pdist L1
  sb::DistanceMatrix<float> viaBlocks(n), viaFactory(n);
  run_blocks<sb::DistanceMatrix<float>, sb::OperationL1Dist<float, float>, sb::DistanceMatrixResultWriter<float>>(
      viaBlocks, dmgr, dmgr, sb::OperationL1Dist<float, float>{}, sb::TriangleSkipMode::LowerTriangleSkipDiag, true);
  auto t = sb::create_cuda_block_integrate_l1_task(viaFactory, pcfs);
  t->start_async(sb::default_executor());
  t->wait();
  for (size_t k = 0; k < viaFactory.storage_count(); ++k) CHECK(viaBlocks.data()[k] == viaFactory.data()[k]);

  // L2 kernel
  sb::SymmetricMatrix<float> kBlocks(n), kFactory(n);
  run_blocks<sb::SymmetricMatrix<float>, sb::OperationL2InnerProduct<float, float>,
             sb::SymmetricMatrixResultWriter<float>>(kBlocks, dmgr, dmgr, sb::OperationL2InnerProduct<float, float>{},
                                                     sb::TriangleSkipMode::LowerTriangle, true);
  auto t2 = sb::create_cuda_block_integrate_l2_kernel_task(kFactory, pcfs);
  t2->start_async(sb::default_executor());
  t2->wait();
  for (size_t k = 0; k < kFactory.storage_count(); ++k) CHECK(kBlocks.data()[k] == kFactory.data()[k]);

  // cdist Lp, p = 3
  std::vector<float> dBlocks(n * m, -1.f), dFactory(n * m);
  sb::DenseMatrixView<float> view(dBlocks.data(), m);
  run_blocks<sb::DenseMatrixView<float>, sb::OperationLpDist<float, float>, sb::DenseResultWriter<float>>(
      view, dmgr, omgr, sb::OperationLpDist<float, float>(3.f), sb::TriangleSkipMode::None, false);
  auto t3 = sb::create_cuda_block_cdist_lp_task(dFactory.data(), pcfs, others, 3.f);
  t3->start_async(sb::default_executor());
  t3->wait();
  for (size_t k = 0; k < n * m; ++k) CHECK(dBlocks[k] == dFactory[k]);

  // the op's argument checks
  bool thrown = false;
  try { sb::OperationLpDist<float, float> bad(0.5f); } catch (const std::invalid_argument&) { thrown = true; }
  CHECK(thrown);
  std::printf("ok\n");
  return 0;
}
