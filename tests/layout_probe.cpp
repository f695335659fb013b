// Prints the size, alignment and member offsets of the types that cross the
// Contest::execute boundary (Plan, PlanNode, ScanNode, JoinNode, ColumnarTable,
// Column, Page, MappedMemory, DataType).  Compiled once against this
// repository's include/plan.h and once against the reference's
// include/plan.h; equal output means a caller built with either header passes
// and receives the same bytes.
#include <cstddef>
#include <cstdio>

#include "plan.h"

#pragma GCC diagnostic ignored "-Winvalid-offsetof"

#define SZ(T) std::printf("%s size %zu align %zu\n", #T, sizeof(T), alignof(T))
#define OFF(T, m) std::printf("%s.%s %zu\n", #T, #m, offsetof(T, m))

int main() {
    SZ(DataType);
    SZ(MappedMemory);
    SZ(ScanNode);
    OFF(ScanNode, base_table_id);
    SZ(JoinNode);
    OFF(JoinNode, build_left);
    OFF(JoinNode, left);
    OFF(JoinNode, right);
    OFF(JoinNode, left_attr);
    OFF(JoinNode, right_attr);
    SZ(PlanNode);
    OFF(PlanNode, data);
    OFF(PlanNode, output_attrs);
    SZ(Page);
    OFF(Page, data);
    SZ(Column);
    OFF(Column, type);
    OFF(Column, pages);
    SZ(ColumnarTable);
    OFF(ColumnarTable, num_rows);
    OFF(ColumnarTable, columns);
    SZ(Plan);
    OFF(Plan, nodes);
    OFF(Plan, inputs);
    OFF(Plan, root);
    std::printf("DataType INT32 %d INT64 %d FP64 %d VARCHAR %d\n", int(DataType::INT32), int(DataType::INT64),
                int(DataType::FP64), int(DataType::VARCHAR));
    std::printf("NodeType HashJoin %d Scan %d\n", int(NodeType::HashJoin), int(NodeType::Scan));
    return 0;
}
