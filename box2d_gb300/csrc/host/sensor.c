/*
 * Sensors of the GB300 step library (sensor.c:43-420 and shape.c:180-205, 1400-1825 in the
 * reference). A sensor shape keeps the sorted list of the shapes it overlapped at the end
 * of the previous step and of this step; the difference gives begin and end touch events.
 *
 * The overlap test of every (sensor, shape) candidate runs on the device at the end of the
 * step (b2gDev_SensorOverlaps: the tree query's category test, the sensor-event flag, the
 * same-body and filter checks, then GJK distance with radii below 10 FLT_EPSILON). The
 * candidate set is every shape whose fat box meets the sensor's box, as the reference's
 * query of its three trees gives; it does not depend on the trees' structure because each
 * sensor's overlaps are sorted by shape id before use. The host then merges the sweep hits,
 * sorts, removes duplicates and emits events in ascending sensor order, as the reference's
 * serial event pass does.
 */
#include "b2g_world.h"

void h_createSensor( h_world* w, h_shape* shape )
{
	h_sensor z;
	memset( &z, 0, sizeof( z ) );
	z.shapeId = shape->id;
	shape->sensorIndex = w->sensors.count;
	h_push( w->sensors, z );
}

void h_freeSensors( h_world* w )
{
	for ( int i = 0; i < w->sensors.count; ++i )
	{
		h_sensor* s = w->sensors.data + i;
		h_free( s->overlaps1 );
		h_free( s->overlaps2 );
		h_free( s->hits );
	}
	h_free( w->sensors );
	h_free( w->sensorBeginEvents );
	h_free( w->sensorEndEvents[0] );
	h_free( w->sensorEndEvents[1] );
}

/* ascending shape id (the reference's b2CompareVisitors), ties by generation so the order
   does not depend on the sort */
static int h_cmpVisitor( const void* a, const void* b )
{
	const h_visitor* va = a;
	const h_visitor* vb = b;
	if ( va->shapeId != vb->shapeId ) return va->shapeId < vb->shapeId ? -1 : 1;
	return ( va->generation > vb->generation ) - ( va->generation < vb->generation );
}

static b2ShapeId h_sensorShapeId( h_world* w, int shapeId, uint16_t generation )
{
	b2ShapeId id = { shapeId + 1, w->worldId, generation };
	return id;
}

void h_overlapSensors( h_world* w, int endIndex )
{
	int n = w->sensors.count;
	w->sensorStep = w->stepIndex;
	if ( n == 0 ) return;
	/* solver.c:1991-2017: the sweeps' sensor hits join the sensors' hit lists */
	if ( w->devReady )
	{
		const int* hits = NULL;
		int hitCount = 0;
		int rc = b2gDev_SensorHits( w->dev, &hits, &hitCount );
		if ( rc != 0 ) h_fail( w, "sensor hits", rc );
		for ( int k = 0; k < hitCount; ++k )
		{
			const h_shape* sensorShape = w->shapes.data + hits[2 * k];
			if ( sensorShape->sensorIndex == B2_NULL_INDEX ) continue;
			h_visitor v = { hits[2 * k + 1], w->shapes.data[hits[2 * k + 1]].generation };
			h_push( w->sensors.data[sensorShape->sensorIndex].hits, v );
		}
	}
	int* query = malloc( (size_t)n * sizeof( int ) );
	unsigned char* changed = calloc( (size_t)n, 1 );
	/* sensor.c:145-175: swap the overlap lists, start the new one with the sweep hits */
	for ( int i = 0; i < n; ++i )
	{
		h_sensor* sensor = w->sensors.data + i;
		h_visitorArray t = sensor->overlaps1;
		sensor->overlaps1 = sensor->overlaps2;
		sensor->overlaps2 = t;
		sensor->overlaps2.count = 0;
		for ( int k = 0; k < sensor->hits.count; ++k ) h_push( sensor->overlaps2, sensor->hits.data[k] );
		sensor->hits.count = 0;
		const h_shape* shape = w->shapes.data + sensor->shapeId;
		const h_body* body = w->bodies.data + shape->bodyId;
		int active = body->setIndex != H_DISABLED_SET && shape->enableSensorEvents;
		query[i] = active ? sensor->shapeId : -1;
		if ( active == 0 && sensor->overlaps1.count != 0 ) changed[i] = 1;
	}
	const int* pairs = NULL;
	int pairCount = 0;
	if ( w->devReady )
	{
		int rc = b2gDev_SensorOverlaps( w->dev, query, n, w->shapes.count, &pairs, &pairCount );
		if ( rc != 0 ) h_fail( w, "sensor overlaps", rc );
	}
	for ( int k = 0; k < pairCount; ++k )
	{
		int sensorIndex = pairs[2 * k], shapeId = pairs[2 * k + 1];
		h_visitor v = { shapeId, w->shapes.data[shapeId].generation };
		h_push( w->sensors.data[sensorIndex].overlaps2, v );
	}
	/* sensor.c:208-248: sort, remove duplicates, compare with the previous step */
	for ( int i = 0; i < n; ++i )
	{
		if ( query[i] < 0 ) continue;
		h_sensor* sensor = w->sensors.data + i;
		h_visitorArray* o2 = &sensor->overlaps2;
		if ( o2->count > 1 ) qsort( o2->data, (size_t)o2->count, sizeof( h_visitor ), h_cmpVisitor );
		int unique = 0;
		for ( int k = 0; k < o2->count; ++k )
			if ( unique == 0 || o2->data[k].shapeId != o2->data[unique - 1].shapeId ) o2->data[unique++] = o2->data[k];
		o2->count = unique;
		const h_visitorArray* o1 = &sensor->overlaps1;
		if ( o1->count != o2->count ) changed[i] = 1;
		else
			for ( int k = 0; k < o1->count; ++k )
				if ( o1->data[k].shapeId != o2->data[k].shapeId || o1->data[k].generation != o2->data[k].generation )
				{
					changed[i] = 1;
					break;
				}
	}
	/* sensor.c:272-385: begin and end events of the sensors that changed, in sensor order */
	for ( int i = 0; i < n; ++i )
	{
		if ( changed[i] == 0 ) continue;
		const h_sensor* sensor = w->sensors.data + i;
		b2ShapeId sensorId = h_sensorShapeId( w, sensor->shapeId, w->shapes.data[sensor->shapeId].generation );
		const h_visitor* r1 = sensor->overlaps1.data;
		const h_visitor* r2 = sensor->overlaps2.data;
		int c1 = sensor->overlaps1.count, c2 = sensor->overlaps2.count;
		int i1 = 0, i2 = 0;
		while ( i1 < c1 || i2 < c2 )
		{
			int end = 0, begin = 0;
			if ( i1 < c1 && i2 < c2 )
			{
				if ( r1[i1].shapeId == r2[i2].shapeId )
				{
					if ( r1[i1].generation < r2[i2].generation ) end = 1;
					else if ( r1[i1].generation > r2[i2].generation ) begin = 1;
					else
					{
						i1 += 1;
						i2 += 1;
						continue;
					}
				}
				else if ( r1[i1].shapeId < r2[i2].shapeId ) end = 1;
				else begin = 1;
			}
			else if ( i1 < c1 ) end = 1;
			else begin = 1;
			if ( end )
			{
				b2SensorEndTouchEvent ev = { sensorId, h_sensorShapeId( w, r1[i1].shapeId, r1[i1].generation ) };
				h_push( w->sensorEndEvents[endIndex], ev );
				i1 += 1;
			}
			else if ( begin )
			{
				b2SensorBeginTouchEvent ev = { sensorId, h_sensorShapeId( w, r2[i2].shapeId, r2[i2].generation ) };
				h_push( w->sensorBeginEvents, ev );
				i2 += 1;
			}
		}
	}
	free( query );
	free( changed );
}

/* ---- public API ---- */

static h_shape* h_sensorShape( b2ShapeId shapeId, h_world** world )
{
	h_world* w = h_worldByIndex( shapeId.world0 );
	*world = w;
	return w->shapes.data + ( shapeId.index1 - 1 );
}

b2SensorEvents b2World_GetSensorEvents( b2WorldId worldId )
{
	h_world* w = h_worldFromId( worldId );
	b2SensorEvents e;
	memset( &e, 0, sizeof( e ) );
	if ( w == NULL || w->locked ) return e;
	/* the step flips the end-event buffers when it ends (physics_world.c:1462-1463) */
	int endIndex = 1 - w->endEventArrayIndex;
	e.beginEvents = w->sensorBeginEvents.data;
	e.beginCount = w->sensorBeginEvents.count;
	e.endEvents = w->sensorEndEvents[endIndex].data;
	e.endCount = w->sensorEndEvents[endIndex].count;
	return e;
}

bool b2Shape_IsSensor( b2ShapeId shapeId )
{
	h_world* w;
	return h_sensorShape( shapeId, &w )->sensorIndex != B2_NULL_INDEX;
}

void b2Shape_EnableSensorEvents( b2ShapeId shapeId, bool flag )
{
	h_world* w;
	h_shape* s = h_sensorShape( shapeId, &w );
	if ( w->locked || s->enableSensorEvents == (int)flag ) return;
	h_markHostChanged( w );
	s->enableSensorEvents = flag;
}

bool b2Shape_AreSensorEventsEnabled( b2ShapeId shapeId )
{
	h_world* w;
	return h_sensorShape( shapeId, &w )->enableSensorEvents != 0;
}

int b2Shape_GetSensorCapacity( b2ShapeId shapeId )
{
	h_world* w;
	h_shape* s = h_sensorShape( shapeId, &w );
	if ( s->sensorIndex == B2_NULL_INDEX ) return 0;
	return w->sensors.data[s->sensorIndex].overlaps2.count;
}

int b2Shape_GetSensorData( b2ShapeId shapeId, b2ShapeId* visitorIds, int capacity )
{
	h_world* w;
	h_shape* s = h_sensorShape( shapeId, &w );
	if ( s->sensorIndex == B2_NULL_INDEX ) return 0;
	const h_sensor* sensor = w->sensors.data + s->sensorIndex;
	int count = sensor->overlaps2.count < capacity ? sensor->overlaps2.count : capacity;
	for ( int i = 0; i < count; ++i )
	{
		b2ShapeId id = { sensor->overlaps2.data[i].shapeId + 1, shapeId.world0, sensor->overlaps2.data[i].generation };
		visitorIds[i] = id;
	}
	return count;
}
