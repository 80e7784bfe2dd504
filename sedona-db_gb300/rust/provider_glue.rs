// provider_glue.rs — the changes to the reference's GPU provider crate
// (rust/sedona-spatial-join-gpu/src/) that route its planner, index and
// geometry factory to this library: ST_DWithin and KNN accepted by the
// planner gate, query_batch through the fused join (one FFI call per batch,
// no host work between filter and refine), query_knn, and distance
// expansion in the evaluated-array factory.  Each section names the file and
// function it replaces.
//
// Not compiled in this repository (there is no Rust toolchain here); the
// types and trait signatures are the reference's at the cited lines.

// ---------------------------------------------------------------------------
// physical_planner.rs:117-157 is_spatial_predicate_supported
//
// Relation predicates as before; ST_DWithin (points, polygons and
// multipolygons, scalar or per-row distance) and KNN (point build and probe
// columns, Euclidean metric) are now on the GPU path.  The library decodes
// Point, Polygon and MultiPolygon rows; when the planner knows a column's
// geometry types (GeoStatistics::geometry_types, from GeoParquet metadata)
// and they include others, the join stays on the CPU, as the reference does
// for unsupported predicates (physical_planner.rs:76-86).

use sedona_expr::statistics::GeoStatistics;
use sedona_geometry::types::GeometryTypeId;

fn types_on_gpu(stats: Option<&GeoStatistics>, points_only: bool) -> bool {
    let Some(types) = stats.and_then(|s| s.geometry_types()) else {
        return true; // unknown: the library reports other types at run time
    };
    types.iter().all(|t| match t.geometry_type() {
        GeometryTypeId::Point => true,
        GeometryTypeId::Polygon | GeometryTypeId::MultiPolygon => !points_only,
        _ => false,
    })
}

pub fn is_spatial_predicate_supported(
    spatial_predicate: &SpatialPredicate,
    left_schema: &Schema,
    right_schema: &Schema,
    left_stats: Option<&GeoStatistics>,
    right_stats: Option<&GeoStatistics>,
) -> Result<bool> {
    fn is_geometry(expr: &Arc<dyn PhysicalExpr>, schema: &Schema) -> Result<bool> {
        let field = expr.return_field(schema)?;
        let sedona_type = SedonaType::from_storage_field(&field)?;
        Ok(ArgMatcher::is_geometry().match_type(&sedona_type))
    }
    let both = |l: &Arc<dyn PhysicalExpr>, r: &Arc<dyn PhysicalExpr>, points_only: bool| -> Result<bool> {
        Ok(is_geometry(l, left_schema)?
            && is_geometry(r, right_schema)?
            && types_on_gpu(left_stats, points_only)
            && types_on_gpu(right_stats, points_only))
    };
    match spatial_predicate {
        SpatialPredicate::Relation(RelationPredicate { left, right, relation_type }) => {
            if !matches!(
                relation_type,
                SpatialRelationType::Intersects
                    | SpatialRelationType::Contains
                    | SpatialRelationType::Within
                    | SpatialRelationType::Covers
                    | SpatialRelationType::CoveredBy
                    | SpatialRelationType::Touches
                    | SpatialRelationType::Equals
            ) {
                return Ok(false);
            }
            both(left, right, false)
        }
        SpatialPredicate::Distance(DistancePredicate { left, right, .. }) => both(left, right, false),
        SpatialPredicate::KNearestNeighbors(KNNPredicate { left, right, use_spheroid, .. }) => {
            Ok(!*use_spheroid && both(left, right, true)?)
        }
    }
}

// ---------------------------------------------------------------------------
// index/gpu_spatial_index.rs:163-229 GPUSpatialIndex::query_batch
//
// One SpjJoin per probe partition (the reference shares one index and one
// refiner between partitions and calls them concurrently; an SpjJoin serves
// one thread at a time, so the builder makes `probe_threads_count` of them,
// each built from the same concatenated build batch, and query_batch takes
// one from a pool).  The probe rows' WKB go in as an Arrow slice; the pairs
// come back refined.

impl GPUSpatialIndex {
    fn predicate_code(&self) -> Result<(i32, Option<f64>)> {
        match &self.spatial_predicate {
            SpatialPredicate::Relation(rel) => {
                Ok((Self::convert_relation_type(&rel.relation_type)? as i32, None))
            }
            SpatialPredicate::Distance(_) => Ok((SPJ_PREDICATE_DWITHIN, Some(0.0))),
            SpatialPredicate::KNearestNeighbors(_) => {
                Err(DataFusionError::Internal("KNN goes through query_knn".into()))
            }
        }
    }

    async fn query_batch_fused(
        &self,
        evaluated_batch: &Arc<EvaluatedBatch>,
        range: Range<usize>,
        build_batch_positions: &mut Vec<(i32, i32)>,
        probe_indices: &mut Vec<u32>,
    ) -> Result<(QueryResultMetrics, usize)> {
        if range.is_empty() {
            return Ok((QueryResultMetrics { count: 0, candidate_count: 0 }, range.start));
        }
        let (predicate, scalar) = self.predicate_code()?;
        let geoms = evaluated_batch
            .geom_array
            .geometry_array()
            .slice(range.start, range.end - range.start);
        let (array, schema) = arrow::ffi::to_ffi(&geoms.to_data())
            .map_err(|e| DataFusionError::Execution(e.to_string()))?;
        let mut join = self.joins.take().await; // a per-partition SpjJoin from the pool
        if predicate == SPJ_PREDICATE_DWITHIN {
            // the evaluated batch carries the probe rows' distances when the
            // distance is a column (operand_evaluator.rs:556-627)
            let distances = evaluated_batch.geom_array.distances_f64(range.clone());
            join.set_probe_distances(distances.as_deref())
                .map_err(DataFusionError::Execution)?;
        }
        let (mut b, mut p) = (Vec::new(), Vec::new());
        join.probe(&schema, &array, predicate, scalar.unwrap_or(0.0), 0, &mut b, &mut p)
            .map_err(|e| DataFusionError::Execution(format!("GPU spatial query failed: {e}")))?;
        self.joins.put(join);
        let count = b.len();
        build_batch_positions.reserve(count);
        probe_indices.reserve(count);
        for (bi, pi) in b.iter().zip(p.iter()) {
            build_batch_positions.push(self.data_id_to_batch_pos[*bi as usize]);
            probe_indices.push(range.start as u32 + pi);
        }
        Ok((QueryResultMetrics { count, candidate_count: count }, range.end))
    }
}

// ---------------------------------------------------------------------------
// index/gpu_spatial_index.rs:252-264 GPUSpatialIndex::query_knn
//
// The reference returns NotImplemented here.  With a point build side the
// builder also makes an SpjKnnHandle over the build points (FP64 xy in
// data-id order); one probe row's WKB goes in as a one-row Arrow array.

impl GPUSpatialIndex {
    fn query_knn_gpu(
        &self,
        probe_wkb: &Wkb,
        k: u32,
        use_spheroid: bool,
        include_tie_breakers: bool,
        build_batch_positions: &mut Vec<(i32, i32)>,
        distances: Option<&mut Vec<f64>>,
    ) -> Result<QueryResultMetrics> {
        if use_spheroid {
            return Err(DataFusionError::NotImplemented(
                "spheroid KNN is not on the GPU path".to_string(),
            ));
        }
        let Some(knn) = self.knn.as_ref() else {
            return Err(DataFusionError::Internal("KNN index not built".into()));
        };
        let one = arrow_array::BinaryArray::from(vec![probe_wkb.buf()]);
        let (array, schema) = arrow::ffi::to_ffi(&one.to_data())
            .map_err(|e| DataFusionError::Execution(e.to_string()))?;
        let (offsets, idx, dist) = knn
            .lock()
            .query(&schema, &array, 1, k, include_tie_breakers)
            .map_err(DataFusionError::Execution)?;
        let (s, e) = (offsets[0] as usize, offsets[1] as usize);
        for i in s..e {
            build_batch_positions.push(self.data_id_to_batch_pos[idx[i] as usize]);
        }
        if let Some(d) = distances {
            d.extend_from_slice(&dist[s..e]);
        }
        Ok(QueryResultMetrics { count: e - s, candidate_count: e - s })
    }
}

// ---------------------------------------------------------------------------
// join_provider.rs:94-145 DefaultGeometryArrayFactory::try_new_evaluated_array
//
// The reference rejects a distance here ("rectangle expansion by distance
// is not yet supported for GPU joins", join_provider.rs:101-104).  The
// library expands the probe rects on the device (from the WKB's exact
// bounds, by each row's distance, rounded outward), so the factory keeps the
// distance with the array and builds the rects as the CPU factory does.

impl EvaluatedGeometryArrayFactory for DefaultGeometryArrayFactory {
    fn try_new_evaluated_array(
        &self,
        geometry_array: ArrayRef,
        sedona_type: &SedonaType,
        distance_columnar_value: Option<&ColumnarValue>,
    ) -> Result<EvaluatedGeometryArray> {
        let mut evaluated = build_rects_as_before(geometry_array, sedona_type)?;
        if let Some(distance) = distance_columnar_value {
            // the rects used by the host-side filter are expanded as the CPU
            // path expands them (operand_evaluator.rs:605-607); the device
            // expands its own copy from the same distances
            evaluated.expand_rects_by(distance)?;
            evaluated.set_distances(distance.clone());
        }
        Ok(evaluated)
    }
}
