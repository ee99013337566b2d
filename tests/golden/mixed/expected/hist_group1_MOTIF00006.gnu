set output "hist_group1_MOTIF00006.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-64.4191:19.6985]
set yrange [0:161632]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_group1_MOTIF00006.dat" using 1:2 title 'MOTIF00006 (group1)' with boxes
