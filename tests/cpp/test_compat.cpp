// Host-only checks of include/sbgpu/compat.hpp (no GPU needed).
//   test_compat schedule nRows nCols maxOut nSplits lower minSide
//       prints "count maxRowHeight maxColWidth" then one block per line
//   test_compat writers
//       runs the result-writer / matrix known-answer checks (restated from
//       the reference's test/test_result_writer.cpp), prints "ok"
#include <sbgpu/compat.hpp>

#include <cstdio>
#include <cstdlib>
#include <cstring>

#define CHECK(c)                                                             \
  do {                                                                       \
    if (!(c)) { std::printf("FAIL %s:%d %s\n", __FILE__, __LINE__, #c); std::exit(1); } \
  } while (0)

template <typename Tv>
static void writer_checks()
{
  {
    sb::DistanceMatrix<Tv> dm(4);
    Tv block[] = {Tv(10), Tv(20), Tv(30), Tv(40)};  // rows 2..3 x cols 0..1
    sb::BlockInfo b{2, 2, 0, 2, 0};
    sb::DistanceMatrixResultWriter<Tv> w(dm);
    w.scatter(block, b);
    CHECK(Tv(dm(2, 0)) == Tv(10) && Tv(dm(2, 1)) == Tv(20) && Tv(dm(3, 0)) == Tv(30) && Tv(dm(3, 1)) == Tv(40));
    CHECK(Tv(dm(0, 2)) == Tv(10));
    CHECK(Tv(dm(1, 0)) == Tv(0) && Tv(dm(2, 3)) == Tv(0));
    CHECK(dm.data()[0] == Tv(0) && dm.data()[1] == Tv(10));  // storage order: (1,0), (2,0), ...
  }
  {
    sb::DistanceMatrix<Tv> dm(4);
    Tv block[] = {Tv(0), Tv(0), Tv(60), Tv(0)};  // diagonal block rows/cols 1..2
    sb::BlockInfo b{1, 2, 1, 2, 0};
    sb::DistanceMatrixResultWriter<Tv> w(dm);
    w.scatter(block, b);
    CHECK(Tv(dm(2, 1)) == Tv(60) && Tv(dm(1, 1)) == Tv(0));
  }
  {
    sb::DistanceMatrix<Tv> dm(4);
    Tv block[] = {Tv(0), Tv(50), Tv(60), Tv(0)};  // (1,2) is above the diagonal and non-zero
    sb::BlockInfo b{1, 2, 1, 2, 0};
    sb::DistanceMatrixResultWriter<Tv> w(dm);
    bool thrown = false;
    try { w.scatter(block, b); } catch (const std::logic_error&) { thrown = true; }
    CHECK(thrown);
  }
  {
    sb::SymmetricMatrix<Tv> sm(3);
    Tv block[] = {Tv(1), Tv(0), Tv(0), Tv(2), Tv(3), Tv(0), Tv(4), Tv(5), Tv(6)};
    sb::BlockInfo b{0, 3, 0, 3, 0};
    sb::SymmetricMatrixResultWriter<Tv> w(sm);
    w.scatter(block, b);
    CHECK(sm(0, 0) == Tv(1) && sm(1, 0) == Tv(2) && sm(1, 1) == Tv(3) && sm(2, 0) == Tv(4) && sm(2, 2) == Tv(6));
    CHECK(sm(0, 2) == Tv(4));
    const Tv want[] = {Tv(1), Tv(2), Tv(3), Tv(4), Tv(5), Tv(6)};  // SymmetricMatrix storage order
    for (int k = 0; k < 6; ++k) CHECK(sm.data()[k] == want[k]);
  }
  {
    std::vector<Tv> dense(2 * 3, Tv(0));
    sb::DenseResultWriter<Tv> w(sb::DenseMatrixView<Tv>(dense.data(), 3));
    Tv block[] = {Tv(7), Tv(8)};
    sb::BlockInfo b{1, 1, 1, 2, 0};
    w.scatter(block, b);
    CHECK(dense[4] == Tv(7) && dense[5] == Tv(8) && dense[0] == Tv(0));
  }
  {
    sb::DistanceMatrix<Tv> dm(3);
    bool neg = false, diag = false;
    try { dm(0, 1) = Tv(-1); } catch (const std::invalid_argument&) { neg = true; }
    try { dm(1, 1) = Tv(2); } catch (const std::invalid_argument&) { diag = true; }
    dm(1, 1) = Tv(0);
    CHECK(neg && diag);
    bool oob = false;
    try { (void)Tv(dm(3, 0)); } catch (const std::out_of_range&) { oob = true; }
    CHECK(oob);
  }
}

int main(int argc, char** argv)
{
  if (argc >= 2 && std::strcmp(argv[1], "writers") == 0)
  {
    writer_checks<float>();
    writer_checks<double>();
    std::printf("ok\n");
    return 0;
  }
  if (argc == 8 && std::strcmp(argv[1], "schedule") == 0)
  {
    sb::CudaBlockScheduler::Config c{};
    c.nRows = std::strtoull(argv[2], nullptr, 10);
    c.nCols = std::strtoull(argv[3], nullptr, 10);
    c.maxOutputElements = std::strtoull(argv[4], nullptr, 10);
    c.nSplitsHint = std::strtoull(argv[5], nullptr, 10);
    c.triangleMode = std::atoi(argv[6]) ? sb::BlockTriangleMode::LowerTriangle : sb::BlockTriangleMode::Full;
    c.minBlockSide = std::strtoull(argv[7], nullptr, 10);
    sb::CudaBlockScheduler s(c);
    std::printf("%zu %zu %zu\n", s.blocks().size(), s.max_row_height(), s.max_col_width());
    for (const auto& b : s.blocks())
      std::printf("%zu %zu %zu %zu %zu\n", b.rowStart, b.rowHeight, b.colStart, b.colWidth, b.blockIndex);
    return 0;
  }
  std::printf("usage: test_compat writers | schedule nRows nCols maxOut nSplits lower minSide\n");
  return 2;
}
